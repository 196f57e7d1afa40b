// Differentiable rollout kernels (forward with checkpoints, backward with recompute).
#pragma once
#include "adjoint_device.cuh"

namespace gbt {

constexpr int kDiffThreads = 256;

// Device buffers of one differentiable rollout.  Colour order = the device element tables' order.
struct DiffBuffers {
    // parameters
    const float* theta;        // [T] per-tet log-compliance, storage order
    const int* slotStorage;    // [T] colour slot -> storage index
    const float2* bake;        // [T] colour order: (mu V, kappa V) the compliance scales
    float young;               // Young's modulus of the bake
    const float* path;         // [(frames + 1) * 6] capsule end points (a, b) per command, or null
    float radius;
    int frames, every, total;  // frames, checkpoint interval (substeps), substeps in all
    const float4* originPos; const float4* originVel;
    // state kept by the forward
    float4* ckPos; float4* ckVel;                 // [segments][N] state before substep seg * every
    // tape of one segment, written by the backward's recompute
    float4* tapeQ; float4* tapeV; float4* tapeX;  // [every][N] substep start, predicted velocity, pre-contact
    float4* tapeEdge;                             // [every][E][2] edge end points before projection
    float4* tapeTet;                              // [every][T][4] tet corners before projection
    // adjoints
    float4* gx; float4* gv; float4* gq;           // [N]
    float* gTheta;                                // [T] storage order
    float* gRest;                                 // [E] colour order, or null
    float* gB;                                    // [T][9] colour order, or null
    float* pathPartial;                           // [total][blocks][6] per-block capsule adjoints
};

__global__ void diffForwardGrid(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b, unsigned* barrier, long long budget);
__global__ void diffForwardBlock(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b);
__global__ void diffBackwardGrid(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b, unsigned* barrier, long long budget);
__global__ void diffBackwardBlock(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b);
// capsule path adjoint from the per-block partials: one thread per (command, component)
__global__ void diffPathGradient(DiffBuffers b, int blocks, int substeps, float* gPath);
// small layout kernels
__global__ void packPositions(int n, const float4* pos, float* out3);
__global__ void unpackGradient(int n, const float* in3, float4* out);
__global__ void scatterSlots(int n, const float* src, const int* slot, float* dst);
__global__ void scatterRows9(int n, const float* src, const int* slot, float* dst);

}  // namespace gbt
