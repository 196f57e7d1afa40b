// Dual-contouring surface of the deformed lattice (V/dc_recon.cu): one persistent launch rebuilds
// the feature point of every surface voxel, stitches the quads of the surface edges, accumulates
// the vertex normals and expands the indexed triangles into a vertex soup.
#pragma once
#include "tissue_device.cuh"

namespace gbt {

// Hermite crossing of one voxel edge (IsectGpu, V/common.cuh:23-32): listed voxel by voxel.
struct IsectRec { float px, py, pz, nx, ny, nz; int a, b; float t; int insideA; };
static_assert(sizeof(IsectRec) == 40, "IsectGpu is 40 bytes");

struct SurfaceMesh {
    int dx, dy, dz;                     // voxel dims
    int nSurfVox, nEdges, triCapacity, qefIters;
    int haveRest;                       // rest feature points exist: intact voxels follow the lattice
    int cutActive;                      // cut buffers present: severed crossings, cut voxels keep the QEF
    const int* surfVox;                 // voxels with a crossing, ascending
    const int* voxelCorner;             // [8V] corner ids, local order (0,0,0) (1,0,0) (1,1,0) (0,1,0) ...
    const int* isectOff; const int* isectCnt; const IsectRec* isect;
    const int4* edges;                  // surface edges: (axis | insideA << 2, base corner x, y, z)
    const float4* pos; const float4* rest;
    const int* nbr; const float* rot; const float* cutT; const unsigned* cutMask;
    float4* fp; const float4* fpRest;   // [V] feature points (w = 1 when set), rest snapshot
    int* nrmFixed;                      // [3V] fixed-point normal sums
    int* tri; unsigned* triCount;       // [3 cap] vertex tags (voxel id, or cut-point slot | 1 << 31
                                        // [| 1 << 30 on cut walls]), 3 x emitted triangles
    int* blockTotal;                    // [2 gridDim] triangles of each CTA's ranges
    // cut voxels (V/cut.cu:761-1100): one feature point per (voxel, corner component)
    int nVox;
    const int* conn;                    // [4096 x 9] component count and component of local corners 0..7
    const unsigned* occupied; const int* inside; const float* skinT; const int* active;
    const float4* cutRec;               // [2 x 6N] cut points per directed lattice slot (owner frame)
    float4* cutFP;                      // [8V] component feature points (w = 1 when set)
    int* cutNrmFixed;                   // [3 x 8V] their fixed-point normal sums
    int* raw;                           // [3 cap] triangles before internal faces cancel
    int4* faces; int faceCap;           // hash table of triangle keys (power of two entries)
    int* wallCount;                     // [V] wall faces of a cut voxel, then the index of its first face (-1: none)
    float* outPos; float* outNrm; float4* outAux;   // [3 cap] vertex soup: xyz, xyz, rest anchor + wall flag
};

constexpr int kSurfaceThreads = 256;
__global__ void surfaceKernel(SurfaceMesh s, unsigned* sync, long long spinBudget);

}  // namespace gbt
