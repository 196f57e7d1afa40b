// Kernels of the frame driver, launched by the host API (lcs_api.cu).
#pragma once
#include "tissue_device.cuh"

namespace gbt {

constexpr int kFrameThreads = 256;     // threads per CTA of the whole-GPU frame kernel
constexpr int kBlockThreads = 512;     // threads of the one-CTA frame kernel

__global__ void frameKernelGrid(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                unsigned* state);
__global__ void frameKernelBlock(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                 unsigned* state);
// the frame of batched instances in lockstep (two CTAs per SM)
__global__ void frameKernelLockstep(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                    unsigned* state);
// the same frames with the tissue guard and contact model 1 compiled in
__global__ void frameKernelGridExt(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                unsigned* state);
__global__ void frameKernelBlockExt(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                 unsigned* state);
// Per-instance view of a packed batch: node range and colour ranges of every instance, and the
// work list of each CTA of frameKernelInstances.
struct InstanceTable {
    const int* nodeBase; const int* nodeCount;
    const int2* edgeRange; const int2* bendRange; const int2* tetRange;   // [instances x colours]
    const int* order; const int* ctaStart;                                 // CTA b: order[ctaStart[b] .. ctaStart[b+1])
    unsigned* derived;                                                     // per instance: revision its liveness was derived at
};
__global__ void frameKernelInstances256(DeviceMesh m, FrameCoeffs fc, ContactParams cp, InstanceTable it);
// Instances on thread-block clusters of 2^logK CTAs x kClusterThreads, positions in distributed
// shared memory (dynamic shared memory: the per-CTA slots of the largest instance, 16 B each);
// it.ctaStart indexes clusters.
constexpr int kClusterThreads = 512, kClusterLogThreads = 9;
__global__ void frameKernelCluster(DeviceMesh m, FrameCoeffs fc, ContactParams cp, InstanceTable it, int logK);
__global__ void frameKernelInstances512(DeviceMesh m, FrameCoeffs fc, ContactParams cp, InstanceTable it);
// A single mesh on one cluster of 2^logK CTAs x kSessionClusterThreads, positions in distributed
// shared memory (plain frames: no blade tick, guard or friction; particle frames by a following
// launch).  256 threads a CTA, so the tet projection keeps its registers.
constexpr int kSessionClusterThreads = 256, kSessionClusterLogThreads = 8;
__global__ void frameKernelSessionCluster(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp,
                                          CutParams cu, unsigned* state, int logK);

__global__ void particleRotKernel(DeviceMesh m, const unsigned* parityWord, int parity);
__global__ void tetAlphaKernel(int n, float invH2, const float2* stiff, float2* alpha);
__global__ void gravityKernel(int n, float gx, float gy, float gz, float4* ext);
// xyz of n float4 records, packed as 3n floats (the getters' host layout)
__global__ void packXyzKernel(int n, const float4* in, float* out);
// 3n packed floats into the xyz of n float4 records, keeping each record's w (inverse mass, mass)
__global__ void unpackXyzKernel(int n, const float* in, float4* out);

struct QuadTool { f3 t1[3], t2[3], lo, hi, ncut; int valid; };
__global__ void detectQuadKernel(DeviceMesh m, CutParams cu, QuadTool tool, const float* rot);
__global__ void severKernel(DeviceMesh m, CutParams cu);
// `barriers` grid barriers and nothing else (the latency floor of a frame phase); sync = {counter, status}
__global__ void barrierFloorKernel(unsigned* sync, int barriers, long long budget);

}  // namespace gbt
