// Dual-contouring surface rebuild (V/dc_recon.cu:97-455 kernels, 469-487 intact advection, 507-541
// pipeline order), as one cooperative launch with grid barriers between its phases:
//   1. feature point of every surface voxel: crossings on the deformed lattice (a severed crossing is
//      rebuilt from its inside particle's frame), then either the advected rest feature point
//      (intact voxels once the rest surface exists) or the QEF gradient walk clamped to the voxel
//      box; the voxel's normal accumulator is cleared;
//   2. stitch: every surface edge's four voxels form a quad, two triangles, degenerate ones dropped.
//      The CTAs own contiguous edge ranges and write at the prefix sum of the ranges before them,
//      so the triangle list is in surface-edge order on every run (the reference appends with an
//      atomic counter, in arrival order);
//      Each written triangle scatters its area-weighted face normal to its vertices as 2^20 fixed
//      point (integer sums: the same result in any order);
//   3. the indexed triangles expanded into the vertex soup the getters return (position, unit
//      normal of the vertex's sum, rest anchor + wall flag).
// Arithmetic follows the reference's expressions and order (no contraction), like the frame
// kernels, so the CPU restatement reproduces every bit.
#include "surface.h"
#include "grid_sync.cuh"

namespace gbt {
namespace {

constexpr float kNormalScale = 1048576.0f;   // NORMAL_SCALE (V/common.cuh)

__device__ __forceinline__ f3 lerp3(f3 a, f3 b, float t) {
    return mk(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t);
}

__device__ __forceinline__ int directedSlot(const SurfaceMesh& s, int a, int b) {
    const int d = b - a, ad = d < 0 ? -d : d;
    const int axis = ad == 1 ? 0 : (ad == s.dx + 1 ? 1 : 2);
    return 6 * a + 2 * axis + (d > 0 ? 1 : 0);
}

// Which side of the crossing owns the skin after a cut between them (SkinOwnerA, V/cut.cuh:16-18).
__device__ __forceinline__ bool skinOwnerA(float skinT, float cutT, int insideA) {
    return cutT >= 0.f && cutT <= 1.f && fabsf(skinT - cutT) > 1e-6f ? skinT < cutT : insideA != 0;
}

// World position of crossing `it` (k_RebuildIsectWorld, V/dc_recon.cu:97-147).
__device__ f3 crossingWorld(const SurfaceMesh& s, const IsectRec& it) {
    const int A = it.a, B = it.b;
    const f3 pa = xyz(s.pos[A]), pb = xyz(s.pos[B]);
    if (s.cutActive) {
        const int nx = s.dx + 1, ny = s.dy + 1;
        const int dxi = B % nx - A % nx, dyi = (B / nx) % ny - (A / nx) % ny, dzi = B / (nx * ny) - A / (nx * ny);
        const int axis = dxi != 0 ? 0 : (dyi != 0 ? 1 : 2);
        const int up = dxi + dyi + dzi > 0 ? 1 : 0;
        if (s.nbr[6 * A + 2 * axis + up] < 0) {   // severed: the missing end from the owner's frame
            const f3 dir = xyz(s.rest[B]) - xyz(s.rest[A]);
            const float cutT = s.cutT ? s.cutT[directedSlot(s, A, B)] : -1.f;
            const bool ownerA = skinOwnerA(it.t, cutT, it.insideA);
            const float* q = s.rot + 9 * (size_t)(ownerA ? A : B);
            const f3 off = mk(q[0] * dir.x + q[1] * dir.y + q[2] * dir.z, q[3] * dir.x + q[4] * dir.y + q[5] * dir.z,
                              q[6] * dir.x + q[7] * dir.y + q[8] * dir.z);
            return ownerA ? lerp3(pa, pa + off, it.t) : lerp3(pb - off, pb, it.t);
        }
    }
    return lerp3(pa, pb, it.t);
}

// Feature point of surface voxel v (k_FeaturePoints V/dc_recon.cu:152-208, k_AdvectIntactSurface
// 469-487: an intact voxel's point is its rest point carried trilinearly by the deformed corners).
__device__ void featurePoint(const SurfaceMesh& s, int v) {
    const int* c = s.voxelCorner + 8 * (size_t)v;
    if (s.haveRest && s.fpRest[v].w >= .5f && !(s.cutActive && s.cutMask && s.cutMask[v] != 0u)) {
        const f3 a = xyz(s.rest[c[0]]), b = xyz(s.rest[c[6]]), r = xyz(s.fpRest[v]);
        const f3 uv = mk(fminf(1.f, fmaxf(0.f, (r.x - a.x) / (b.x - a.x))), fminf(1.f, fmaxf(0.f, (r.y - a.y) / (b.y - a.y))),
                         fminf(1.f, fmaxf(0.f, (r.z - a.z) / (b.z - a.z))));
        f3 p = mk(0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const bool x = k == 1 || k == 2 || k == 5 || k == 6, y = k == 2 || k == 3 || k == 6 || k == 7, z = k >= 4;
            const float w = (x ? uv.x : 1.f - uv.x) * (y ? uv.y : 1.f - uv.y) * (z ? uv.z : 1.f - uv.z);
            p = p + xyz(s.pos[c[k]]) * w;
        }
        s.fp[v] = make_float4(p.x, p.y, p.z, 1.f);
        return;
    }
    const int off = s.isectOff[v], cnt = s.isectCnt[v];
    if (cnt <= 0) { s.fp[v] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    f3 world[12];
    f3 x = mk(0.f, 0.f, 0.f);
    for (int k = 0; k < cnt && k < 12; k++) { world[k] = crossingWorld(s, s.isect[off + k]); x = x + world[k]; }
    x = mk(x.x / (float)cnt, x.y / (float)cnt, x.z / (float)cnt);
    f3 lo = xyz(s.pos[c[0]]), hi = lo;
    for (int k = 1; k < 8; k++) {
        const f3 p = xyz(s.pos[c[k]]);
        lo = mk(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
        hi = mk(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
    }
    for (int it = 0; it < s.qefIters; it++) {
        f3 F = mk(0.f, 0.f, 0.f);
        for (int k = 0; k < cnt && k < 12; k++) {
            const IsectRec& rec = s.isect[off + k];
            const f3 n = mk(rec.nx, rec.ny, rec.nz);
            F = F + n * dot(n, world[k] - x);
        }
        const float a = 0.1f * (1.0f - (float)it / (float)s.qefIters);
        const f3 xn = x + F * a;
        if (xn.x <= lo.x || xn.y <= lo.y || xn.z <= lo.z || xn.x >= hi.x || xn.y >= hi.y || xn.z >= hi.z) break;
        x = xn;
    }
    s.fp[v] = make_float4(x.x, x.y, x.z, 1.f);
}

__device__ __forceinline__ f3 fpAt(const SurfaceMesh& s, int v) { return xyz(s.fp[v]); }

// The quad of surface edge e as two triangles (k_Stitch, V/dc_recon.cu:241-289): voxel stencil
// counter-clockwise about +axis, flipped when the base corner is outside; a triangle whose area
// vector is below 1e-8 is dropped.
__device__ void stitchEdge(const SurfaceMesh& s, int e, int ids[6], bool ok[2]) {
    const int4 r = s.edges[e];
    const int axis = r.x & 3, insideA = r.x >> 2;
    int ox[4], oy[4], oz[4];
    if (axis == 0) { ox[0] = 0; oy[0] = 0; oz[0] = 0; ox[1] = 0; oy[1] = -1; oz[1] = 0; ox[2] = 0; oy[2] = -1; oz[2] = -1; ox[3] = 0; oy[3] = 0; oz[3] = -1; }
    else if (axis == 1) { ox[0] = 0; oy[0] = 0; oz[0] = 0; ox[1] = 0; oy[1] = 0; oz[1] = -1; ox[2] = -1; oy[2] = 0; oz[2] = -1; ox[3] = -1; oy[3] = 0; oz[3] = 0; }
    else { ox[0] = 0; oy[0] = 0; oz[0] = 0; ox[1] = -1; oy[1] = 0; oz[1] = 0; ox[2] = -1; oy[2] = -1; oz[2] = 0; ox[3] = 0; oy[3] = -1; oz[3] = 0; }
    int v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = (r.y + ox[k]) + s.dx * ((r.z + oy[k]) + s.dy * (r.w + oz[k]));
    int a = v[0], b = v[1], c = v[2], d = v[3];
    if (insideA == 0) { const int t = b; b = d; d = t; }
    ids[0] = a; ids[1] = b; ids[2] = c; ids[3] = a; ids[4] = c; ids[5] = d;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const f3 p0 = fpAt(s, ids[3 * k]), p1 = fpAt(s, ids[3 * k + 1]), p2 = fpAt(s, ids[3 * k + 2]);
        const f3 n = cross(p1 - p0, p2 - p0);
        ok[k] = !(dot(n, n) < 1e-16f);
    }
}

// Sum over the CTA (every thread calls it).
__device__ int blockSum(int v) {
    __shared__ int partial[kSurfaceThreads / 32];
    __shared__ int total;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) partial[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += partial[w];
        total = t;
    }
    __syncthreads();
    const int out = total;
    __syncthreads();
    return out;
}

// Exclusive prefix of v over the CTA in thread order; *sum receives the CTA total.
__device__ int blockExclusive(int v, int* sum) {
    __shared__ int warpTotal[kSurfaceThreads / 32];
    __shared__ int total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += n;
    }
    if (lane == 31) warpTotal[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { const int x = warpTotal[w]; warpTotal[w] = t; t += x; }
        total = t;
    }
    __syncthreads();
    const int out = warpTotal[warp] + inc - v;
    *sum = total;
    __syncthreads();
    return out;
}

}  // namespace

__global__ void __launch_bounds__(kSurfaceThreads) surfaceKernel(SurfaceMesh s, unsigned* sync, long long spinBudget) {
    GridSync g{sync, sync + 1, gridDim.x, 0u, spinBudget, 0u};
    const int r = g.rank(), R = g.size();
    // 1. feature points; normal accumulators cleared
    for (int j = r; j < s.nSurfVox; j += R) {
        const int v = s.surfVox[j];
        featurePoint(s, v);
        s.nrmFixed[3 * v] = 0; s.nrmFixed[3 * v + 1] = 0; s.nrmFixed[3 * v + 2] = 0;
    }
    if (!g.sync()) return;
    // 2. stitch, in surface-edge order
    const int chunk = (s.nEdges + (int)gridDim.x - 1) / (int)gridDim.x;
    const int e0 = min(s.nEdges, (int)blockIdx.x * chunk), e1 = min(s.nEdges, e0 + chunk);
    int mine = 0;
    for (int e = e0 + (int)threadIdx.x; e < e1; e += blockDim.x) {
        int ids[6]; bool ok[2];
        stitchEdge(s, e, ids, ok);
        mine += (ok[0] ? 1 : 0) + (ok[1] ? 1 : 0);
    }
    const int own = blockSum(mine);
    if (threadIdx.x == 0) s.blockTotal[blockIdx.x] = own;
    if (!g.sync()) return;
    int before = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) before += *(volatile int*)(s.blockTotal + b);
    before = blockSum(before);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *s.triCount = 3u * (unsigned)min(before + own, s.triCapacity);
    int running = before;
    for (int base = e0; base < e1; base += blockDim.x) {
        const int e = base + (int)threadIdx.x;
        int ids[6] = {0, 0, 0, 0, 0, 0};
        bool ok[2] = {false, false};
        if (e < e1) stitchEdge(s, e, ids, ok);
        int roundTotal = 0;
        int t = running + blockExclusive((ok[0] ? 1 : 0) + (ok[1] ? 1 : 0), &roundTotal);
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if (!ok[k]) continue;
            if (t < s.triCapacity) {   // kept triangles scatter their face normal (k_NormalsScatter, V/dc_recon.cu:321-355)
                const int a = ids[3 * k], b = ids[3 * k + 1], c = ids[3 * k + 2];
                s.tri[3 * t] = a; s.tri[3 * t + 1] = b; s.tri[3 * t + 2] = c;
                const f3 p0 = fpAt(s, a), n = cross(fpAt(s, b) - p0, fpAt(s, c) - p0);
                const int fx = (int)(n.x * kNormalScale), fy = (int)(n.y * kNormalScale), fz = (int)(n.z * kNormalScale);
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    const int v = ids[3 * k + q];
                    atomicAdd(s.nrmFixed + 3 * v, fx); atomicAdd(s.nrmFixed + 3 * v + 1, fy); atomicAdd(s.nrmFixed + 3 * v + 2, fz);
                }
            }
            t++;
        }
        running += roundTotal;
    }
    if (!g.sync()) return;
    // 3. vertex soup (k_ExpandVertices V/dc_recon.cu:363-400, external vertices), each vertex's unit
    // normal formed from its fixed-point sum (k_NormalsNormalize, 442-455)
    const int nTri = (int)(*(volatile unsigned*)s.triCount / 3u);
    for (int i = r; i < 3 * nTri; i += R) {
        const int v = s.tri[i];
        const float4 p = s.fp[v], q = s.fpRest[v];
        const f3 n = mk((float)s.nrmFixed[3 * v] / kNormalScale, (float)s.nrmFixed[3 * v + 1] / kNormalScale,
                        (float)s.nrmFixed[3 * v + 2] / kNormalScale);
        const float l = len(n);
        const f3 u = l > 1e-6f ? mk(n.x / l, n.y / l, n.z / l) : mk(0.f, 0.f, 0.f);
        s.outPos[3 * i] = p.x; s.outPos[3 * i + 1] = p.y; s.outPos[3 * i + 2] = p.z;
        s.outNrm[3 * i] = u.x; s.outNrm[3 * i + 1] = u.y; s.outNrm[3 * i + 2] = u.z;
        s.outAux[i] = make_float4(q.x, q.y, q.z, 0.f);
    }
}

}  // namespace gbt
