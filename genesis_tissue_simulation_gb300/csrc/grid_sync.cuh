// Barriers of the persistent kernels.
//   GridSync   cooperative launch over the whole GPU: software grid barrier with a bounded spin
//   BlockSync  one CTA: __syncthreads
// Both expose the participating thread's rank and the team size, so one kernel body serves both.
#pragma once
#include <cuda_runtime.h>

namespace gbt {

// Grid barrier on a monotonically increasing arrival counter (reset by the host before launch).
// After the block's __syncthreads, one thread arrives with a gpu-scope release reduction
// (cumulative: it carries the block's writes), spins on gpu-scope acquire loads with a clock budget, and the
// second __syncthreads hands the acquired view to the block.  A barrier that times out records
// kSyncTimeout in the status word; every block leaves at its next barrier, so the launch ends and
// the host reports the error.
constexpr unsigned kSyncTimeout = 1u;

struct GridSync {
    unsigned* counter; unsigned* status; unsigned nblocks; unsigned target;
    long long budget;     // spin budget in SM clock cycles
    unsigned extra;       // arrivals awaited beyond the grid (non-zero only in the timeout test mode)
    __device__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    // Element-to-thread map of the frame kernels: warp w of CTA b takes logical warp w * gridDim + b,
    // so a phase with fewer elements than threads (a colour of a single mesh) spreads them over every
    // SM instead of packing them into the first CTAs; a warp still takes 32 consecutive elements.
    __device__ int spreadRank() const {
        return (((int)(threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x) << 5) | (int)(threadIdx.x & 31);
    }
    __device__ int size() const { return gridDim.x * blockDim.x; }
    __device__ bool leader() const { return blockIdx.x == 0 && threadIdx.x == 0; }
    __device__ bool sync() {
        __shared__ unsigned ok;
        __syncthreads();
        target += nblocks;
        if (threadIdx.x == 0) {
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" :: "l"(counter) : "memory");
            long long start = clock64();
            for (unsigned polls = 1;; polls++) {
                unsigned now;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(now) : "l"(counter) : "memory");
                if ((int)(now - (target + extra)) >= 0) break;
                // the status word and the clock are looked at every 64th poll (a poll per
                // iteration costs the barrier ~5 %)
                if ((polls & 63u) == 0u) {
                    if (*(volatile unsigned*)status != 0u) break;
                    if (clock64() - start > budget) { atomicOr(status, kSyncTimeout); break; }
                }
            }
            ok = *(volatile unsigned*)status == 0u;
        }
        __syncthreads();
        return ok != 0u;
    }
};

struct BlockSync {
    unsigned* status;
    __device__ int rank() const { return threadIdx.x; }
    __device__ int spreadRank() const { return threadIdx.x; }
    __device__ int size() const { return blockDim.x; }
    __device__ bool sync() { __syncthreads(); return true; }
    __device__ bool leader() const { return threadIdx.x == 0; }
};

}  // namespace gbt
