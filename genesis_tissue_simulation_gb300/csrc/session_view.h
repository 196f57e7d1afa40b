// What other translation units of the library may read of the LCS session (internal, not exported).
#pragma once
#include "tissue_device.cuh"

namespace gbt {

struct SessionView {
    DeviceMesh mesh;                   // device tables of the session (tetAlpha = the session's own)
    cudaStream_t stream;
    int device, smCount, clockKHz, launchMode;
    int N, E, T, numSubsteps;
    float ks, betaS, kb, strainDamping, omega, damping, alpha, youngE, syncBudgetSeconds;
    bool cutActive;                    // a blade is set on an initialised cut: the topology may change
    int volumePasses;                  // tissue guard armed (> 0)
    int contactModel;
    ContactParams cp;
    const int* tetColorOrder;          // host [T]: colour slot -> storage index
    unsigned* state;                   // device: [0] liveness revision, [1] barrier counter, [2] status
    unsigned long long generation;     // changes with every new physics session, cut module and restored state
    const unsigned* revision;          // device: links severed since the cut module was set up (null without one)
};

// 0 and the view when physics is initialised, else a negative status.
int sessionView(SessionView* v);

// Frees the cut-topology product's device buffers (cut_topology.cu); called when a session ends.
void releaseCutTopology();

}  // namespace gbt
