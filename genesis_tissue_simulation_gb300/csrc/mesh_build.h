// Host-side construction of one tissue mesh's solver topology, in the device layout of
// tissue_device.cuh: lattice edges, bend elements and Kuhn tets, each greedily coloured in the
// reference's emission order (xpbd_bind / xpbd_init / xpbd_set_bending / xpbd_build_tets,
// V/xpbd/xpbd_solver.cu:1204-1279, 1332-1400, 1412-1577, 1600-1848) and stored colour-major.
// Used by the single-session C ABI and by the batched instance table.
#pragma once
#include <vector>
#include <cuda_runtime.h>

namespace gbt {

struct MeshInput {
    int dx, dy, dz;                        // voxel dims; nodes (dx+1)(dy+1)(dz+1)
    const float* restPos;                  // [3N] rest lattice (also the initial positions)
    const float* mass; const int* pinned; const int* active; const float* extForce;   // [N], [3N]
    const int* nbrIdx; const float* restNbr;                                          // [6N], [18N]
    const void* bendPairs; int bendPairCount;                                         // 32-byte records
    float youngE, poisson;                 // bake of mu*V and kappa*V
};

struct HostMesh {
    int N = 0, E = 0, B = 0, T = 0;
    std::vector<int> edgeColorOff, bendColorOff, tetColorOff;        // [colours + 1]
    std::vector<int2> edgeEnds; std::vector<float> edgeRest; std::vector<int> edgeOwner;
    std::vector<int4> bendIJK; std::vector<int> bendSrc;
    std::vector<int4> tetIds; std::vector<int> tetMeta, tetOwner; std::vector<float2> tetStiff;   // colour order
    std::vector<int> tetColorOrder;        // colour slot -> storage index (Kuhn type major, cell minor)
    std::vector<int> tetIdsStorage;        // [4T] storage order
    std::vector<float2> tetStiffStorage;   // [T] storage order
    std::vector<float4> pos, ext;          // pos.w = inverse mass, ext.w = mass
    float typeB[6][9];                     // rest Dm^-1 per Kuhn type
};

// Returns 0, or XPBD_ERR_BAD_ARG / XPBD_ERR_COLOR_OVERFLOW / XPBD_ERR_IRREGULAR_REST.
int buildHostMesh(const MeshInput& in, HostMesh& out);

}  // namespace gbt
