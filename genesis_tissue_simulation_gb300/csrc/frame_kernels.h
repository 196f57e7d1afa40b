// Kernels of the frame driver, launched by the host API (lcs_api.cu).
#pragma once
#include "tissue_device.cuh"

namespace gbt {

constexpr int kFrameThreads = 256;     // threads per CTA of both frame kernels

__global__ void frameKernelGrid(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                unsigned* state);
__global__ void frameKernelBlock(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to, ContactParams cp, CutParams cu,
                                 unsigned* state);
__global__ void tetAlphaKernel(int n, float invH2, const float2* stiff, float2* alpha);
__global__ void gravityKernel(int n, float gx, float gy, float gz, float4* ext);

struct QuadTool { f3 t1[3], t2[3], lo, hi; int valid; };
__global__ void detectQuadKernel(DeviceMesh m, CutParams cu, QuadTool tool);
__global__ void severKernel(DeviceMesh m, CutParams cu);

}  // namespace gbt
