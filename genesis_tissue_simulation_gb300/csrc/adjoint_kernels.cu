// Differentiable XPBD rollout: forward with checkpoints, backward by recompute and reverse sweep.
//
// The forward runs every frame of the rollout in one persistent launch, with the projections of the
// plain frame kernel (applyEdge, applyTet) and the capsule contact of the shaft, and stores the node
// state (positions, velocities) every `every` substeps.  The backward walks the segments between
// checkpoints from the last to the first; for each it restores the checkpoint, recomputes the
// segment while recording a tape (substep-start positions, predicted velocities, pre-contact
// positions, and every element's node positions just before its projection), then runs the
// substeps in reverse: velocity and contact, tet colours last to first, edge colours last to
// first, predict.  Elements of one colour touch disjoint nodes in reverse as in forward, so the
// node adjoints need no atomics, and every per-tet and per-edge adjoint is accumulated by a single
// thread in substep order.
#include "adjoint_kernels.h"
#include "grid_sync.cuh"

namespace gbt {

namespace {

__device__ __forceinline__ FrameCoeffs frameCoeffs(const DiffCoeffs& dc) {
    FrameCoeffs fc{};
    fc.alphaTilde = dc.alphaTilde; fc.betaGammaHS = dc.betaGammaHS; fc.omega = dc.omega;
    fc.dampingOverH = dc.dampingOverH; fc.fallback = 0; fc.fallbackInvEh2 = 0.f;
    fc.invScale = 1.f / (1.f + fc.dampingOverH); fc.invBulkScale = fc.invScale;
    return fc;
}

// Capsule of global substep g: frame f lerps command f -> f + 1 at t = (s + 1) / N.
__device__ __forceinline__ Capsule capsuleAt(const DiffBuffers& b, const DiffCoeffs& dc, int g, int N) {
    int f = g / N, s = g - f * N;
    float t = fminf(1.f, (float)(s + 1) / (float)N);
    const float* a = b.path + 6 * f;
    const float* c = b.path + 6 * (f + 1);
    Capsule k;
    k.sa = lerpTool(a[0], a[1], a[2], c[0], c[1], c[2], t);
    k.sb = lerpTool(a[3], a[4], a[5], c[3], c[4], c[5], t);
    k.radius = b.radius;
    k.alpha = dc.contactAlphaH2;
    return k;
}

__device__ __forceinline__ float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }

// One substep forward; with `record`, writes tape slot j.
template <class Sync>
__device__ bool substepForward(const DeviceMesh& m, const DiffCoeffs& dc, const ContactParams& cp, const DiffBuffers& b, int g, int N,
                               bool record, int j, Sync& sync) {
    const int r = sync.spreadRank(), R = sync.size();   // spread: a phase smaller than the grid reaches every SM
    const FrameCoeffs fc = frameCoeffs(dc);
    const int nodes = m.nNodes;
    for (int i = r; i < nodes; i += R) {
        float4 P = m.pos[i];
        m.prev[i] = make_float4(P.x, P.y, P.z, 0.f);
        float4 V = m.vel[i];
        if (P.w > 0.f) {
            float4 Fe = m.ext[i];
            f3 a = mk(Fe.x, Fe.y, Fe.z) * P.w;
            f3 v = xyz(V) + a * dc.h;
            V = make_float4(v.x, v.y, v.z, 0.f);
            m.vel[i] = V;
            f3 x = xyz(P) + v * dc.h;
            m.pos[i] = make_float4(x.x, x.y, x.z, P.w);
        }
        if (record) { b.tapeQ[(size_t)j * nodes + i] = P; b.tapeV[(size_t)j * nodes + i] = V; }
    }
    if (!sync.sync()) return false;
    if (dc.doEdges)
        for (int c = 0; c < m.nEdgeColors; c++) {
            int2 rg = m.edgeRange[c];
            for (int e = rg.x + r; e < rg.y; e += R) {
                EdgeRecord rec = loadEdge(m, e, fc);
                if (record && rec.live) {
                    float4* t = b.tapeEdge + 2 * ((size_t)j * (m.edgeRange[m.nEdgeColors - 1].y) + e);
                    t[0] = m.pos[rec.ij.x]; t[1] = m.pos[rec.ij.y];
                }
                applyEdge(m, rec, fc);
            }
            if (!sync.sync()) return false;
        }
    if (dc.doStrain)
        for (int c = 0; c < m.nTetColors; c++) {
            int2 rg = m.tetRange[c];
            for (int k = rg.x + r; k < rg.y; k += R) {
                TetRecord rec = loadTet(m, k, fc);
                if (record && (rec.meta & 8)) {
                    float4* t = b.tapeTet + 4 * ((size_t)j * (m.tetRange[m.nTetColors - 1].y) + k);
                    t[0] = m.pos[rec.ids.x]; t[1] = m.pos[rec.ids.y]; t[2] = m.pos[rec.ids.z]; t[3] = m.pos[rec.ids.w];
                }
                applyTet(m, rec, fc);
            }
            if (!sync.sync()) return false;
        }
    Capsule cap{};
    if (dc.contact) cap = capsuleAt(b, dc, g, N);
    for (int i = r; i < nodes; i += R) {
        float4 P = m.pos[i];
        if (record) b.tapeX[(size_t)j * nodes + i] = P;
        f3 x = xyz(P);
        if (dc.contact) x = capsuleContact(x, P.w, xyz(m.vel[i]), cap, cp);
        m.pos[i] = f4(x, P.w);
        f3 q = xyz(m.prev[i]);
        f3 v = P.w > 0.f ? (x - q) * dc.invH : mk(0.f, 0.f, 0.f);
        v = P.w > 0.f ? v * dc.velScale : mk(0.f, 0.f, 0.f);
        m.vel[i] = f4(v, 0.f);
    }
    return true;
}

template <class Sync>
__device__ void rolloutForward(const DeviceMesh& m, const DiffCoeffs& dc, const ContactParams& cp, const DiffBuffers& b, int N, Sync& sync) {
    const int r = sync.spreadRank(), R = sync.size();   // spread: a phase smaller than the grid reaches every SM
    // liveness of the current topology, per-tet compliance, origin state with inverse masses
    for (int c = 0; c < m.nEdgeColors; c++)
        for (int e = m.edgeRange[c].x + r; e < m.edgeRange[c].y; e += R) refreshEdge(m, e);
    for (int c = 0; c < m.nTetColors; c++)
        for (int k = m.tetRange[c].x + r; k < m.tetRange[c].y; k += R) {
            refreshTet(m, k);
            m.tetAlpha[k] = tetAlphaFromLog(b.theta[b.slotStorage[k]], b.young, b.bake[k], dc.invH2);
        }
    for (int i = r; i < m.nNodes; i += R) {
        float4 P = b.originPos[i];
        P.w = nodeInvMass(m, i);
        m.pos[i] = P;
        m.vel[i] = b.originVel[i];
    }
    if (!sync.sync()) return;
    for (int g = 0; g < b.total; g++) {
        if (g % b.every == 0) {
            size_t base = (size_t)(g / b.every) * m.nNodes;
            for (int i = r; i < m.nNodes; i += R) { b.ckPos[base + i] = m.pos[i]; b.ckVel[base + i] = m.vel[i]; }
        }
        if (!substepForward(m, dc, cp, b, g, N, false, 0, sync)) return;
    }
}

// Sum of six floats over the block, deterministic (fixed lanes and warps); thread 0 gets it.
__device__ void blockSum6(float v[6], float* out) {
    __shared__ float part[32][6];
#pragma unroll
    for (int c = 0; c < 6; c++)
        for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int c = 0; c < 6; c++) part[warp][c] = v[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        int warps = (blockDim.x + 31) >> 5;
        for (int c = 0; c < 6; c++) {
            float s = 0.f;
            for (int w = 0; w < warps; w++) s += part[w][c];
            out[c] = s;
        }
    }
    __syncthreads();
}

template <class Sync>
__device__ void rolloutBackward(const DeviceMesh& m, const DiffCoeffs& dc, const ContactParams& cp, const DiffBuffers& b, int N, Sync& sync) {
    const int r = sync.spreadRank(), R = sync.size();   // spread: a phase smaller than the grid reaches every SM
    const int nodes = m.nNodes;
    const int E = m.nEdgeColors > 0 ? m.edgeRange[m.nEdgeColors - 1].y : 0;
    const int T = m.nTetColors > 0 ? m.tetRange[m.nTetColors - 1].y : 0;
    const int blocks = gridDim.x;
    const f3 zero = mk(0.f, 0.f, 0.f);
    const int segments = (b.total + b.every - 1) / b.every;
    for (int seg = segments - 1; seg >= 0; seg--) {
        const int g0 = seg * b.every, g1 = min(b.total, g0 + b.every);
        size_t base = (size_t)seg * nodes;
        for (int i = r; i < nodes; i += R) { m.pos[i] = b.ckPos[base + i]; m.vel[i] = b.ckVel[base + i]; }
        if (!sync.sync()) return;
        for (int g = g0; g < g1; g++)
            if (!substepForward(m, dc, cp, b, g, N, true, g - g0, sync)) return;
        if (!sync.sync()) return;
        for (int g = g1 - 1; g >= g0; g--) {
            const int j = g - g0;
            const float4* tq = b.tapeQ + (size_t)j * nodes;
            // velocity update and contact, in reverse
            Capsule cap{};
            if (dc.contact) cap = capsuleAt(b, dc, g, N);
            float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int i = r; i < nodes; i += R) {
                float w = tq[i].w;
                f3 gx = xyz(b.gx[i]), gqv = zero;
                if (w > 0.f) {
                    f3 t = (xyz(b.gv[i]) * dc.velScale) * dc.invH;
                    gx = gx + t;
                    gqv = zero - t;
                }
                if (dc.contact) {
                    f3 gsa = zero, gsb = zero;
                    gx = capsuleContactVJP(xyz(b.tapeX[(size_t)j * nodes + i]), w, xyz(b.tapeV[(size_t)j * nodes + i]), cap, cp, gx, gsa, gsb);
                    acc[0] += gsa.x; acc[1] += gsa.y; acc[2] += gsa.z; acc[3] += gsb.x; acc[4] += gsb.y; acc[5] += gsb.z;
                }
                b.gx[i] = f4(gx, 0.f);
                b.gq[i] = f4(gqv, 0.f);
            }
            if (dc.contact) blockSum6(acc, b.pathPartial + ((size_t)g * blocks + blockIdx.x) * 6);
            if (!sync.sync()) return;
            // tets, last colour first
            if (dc.doStrain)
                for (int c = m.nTetColors - 1; c >= 0; c--) {
                    int2 rg = m.tetRange[c];
                    for (int k = rg.x + r; k < rg.y; k += R) {
                        int meta = m.tetMeta[k];
                        if ((meta & 8) == 0) continue;
                        int4 ids = m.tetIds[k];
                        int id[4] = {ids.x, ids.y, ids.z, ids.w};
                        const float4* t = b.tapeTet + 4 * ((size_t)j * T + k);
                        float4 P[4] = {t[0], t[1], t[2], t[3]};
                        f3 q[4], go[4];
#pragma unroll
                        for (int n = 0; n < 4; n++) { q[n] = xyz(tq[id[n]]); go[n] = xyz(b.gx[id[n]]); }
                        float2 a = m.tetAlpha[k];
                        // what the writes below add to, read before the VJP so its latency overlaps
                        f3 gq0[4];
#pragma unroll
                        for (int n = 0; n < 4; n++) gq0[n] = xyz(b.gq[id[n]]);
                        const int st = b.slotStorage[k];
                        const float th0 = b.gTheta[st];
                        TetAdjoint adj;
                        tetVJP(m.typeB[meta & 7], P, q, a.x, a.y, dc.dampingOverH, dc.omega, go, b.gB != nullptr, adj);
#pragma unroll
                        for (int n = 0; n < 4; n++) {
                            b.gx[id[n]] = f4(adj.gp[n], 0.f);
                            b.gq[id[n]] = f4(gq0[n] + adj.gq[n], 0.f);
                        }
                        b.gTheta[st] = th0 + (adj.gad * a.x + adj.gah * a.y);
                        if (b.gB) {
                            float* gb = b.gB + (size_t)9 * k;
#pragma unroll
                            for (int n = 0; n < 9; n++) gb[n] += adj.gB[n];
                        }
                    }
                    if (!sync.sync()) return;
                }
            // edges, last colour first
            if (dc.doEdges)
                for (int c = m.nEdgeColors - 1; c >= 0; c--) {
                    int2 rg = m.edgeRange[c];
                    for (int e = rg.x + r; e < rg.y; e += R) {
                        if (m.edgeLive[e] == 0) continue;
                        int2 ij = m.edgeEnds[e];
                        const float4* t = b.tapeEdge + 2 * ((size_t)j * E + e);
                        EdgeAdjoint adj = edgeVJP(t[0], t[1], xyz(tq[ij.x]), xyz(tq[ij.y]), m.edgeRest[e], dc.alphaTilde,
                                                  dc.betaGammaHS, dc.omega, xyz(b.gx[ij.x]), xyz(b.gx[ij.y]));
                        b.gx[ij.x] = f4(adj.gpi, 0.f);
                        b.gx[ij.y] = f4(adj.gpj, 0.f);
                        if (dc.betaGammaHS != 0.f) {
                            b.gq[ij.x] = f4(xyz(b.gq[ij.x]) + adj.gqi, 0.f);
                            b.gq[ij.y] = f4(xyz(b.gq[ij.y]) + adj.gqj, 0.f);
                        }
                        if (b.gRest) b.gRest[e] += adj.grest;
                    }
                    if (!sync.sync()) return;
                }
            // predict: x1 = x + h v1, v1 = v + h a, prev = x
            for (int i = r; i < nodes; i += R) {
                float w = tq[i].w;
                f3 g1 = xyz(b.gx[i]);
                b.gv[i] = f4(w > 0.f ? g1 * dc.h : zero, 0.f);
                b.gx[i] = f4(g1 + xyz(b.gq[i]), 0.f);
            }
        }
        if (!sync.sync()) return;
    }
}

}  // namespace

__global__ void __launch_bounds__(kDiffThreads) diffForwardGrid(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b,
                                                                unsigned* barrier, long long budget) {
    GridSync g{barrier, barrier + 1, gridDim.x, 0u, budget, 0u};
    rolloutForward(m, dc, cp, b, b.total / b.frames, g);
}
__global__ void __launch_bounds__(kDiffThreads) diffForwardBlock(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b) {
    BlockSync s{nullptr};
    rolloutForward(m, dc, cp, b, b.total / b.frames, s);
}
__global__ void __launch_bounds__(kDiffThreads) diffBackwardGrid(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b,
                                                                 unsigned* barrier, long long budget) {
    GridSync g{barrier, barrier + 1, gridDim.x, 0u, budget, 0u};
    rolloutBackward(m, dc, cp, b, b.total / b.frames, g);
}
__global__ void __launch_bounds__(kDiffThreads) diffBackwardBlock(DeviceMesh m, DiffCoeffs dc, ContactParams cp, DiffBuffers b) {
    BlockSync s{nullptr};
    rolloutBackward(m, dc, cp, b, b.total / b.frames, s);
}

__global__ void diffPathGradient(DiffBuffers b, int blocks, int substeps, float* gPath) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 6 * (b.frames + 1)) return;
    int pose = idx / 6, c = idx - 6 * pose;
    float acc = 0.f;
    // pose p is the "to" end of frame p - 1 (weight t) and the "from" end of frame p (weight 1 - t)
    for (int f = pose - 1; f <= pose; f++) {
        if (f < 0 || f >= b.frames) continue;
        for (int s = 0; s < substeps; s++) {
            int g = f * substeps + s;
            float t = fminf(1.f, (float)(s + 1) / (float)substeps);
            float sum = 0.f;
            for (int k = 0; k < blocks; k++) sum += b.pathPartial[((size_t)g * blocks + k) * 6 + c];
            acc += sum * (f == pose ? 1.f - t : t);
        }
    }
    gPath[idx] = acc;
}

__global__ void packPositions(int n, const float4* pos, float* out3) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    out3[3 * i] = p.x; out3[3 * i + 1] = p.y; out3[3 * i + 2] = p.z;
}
__global__ void unpackGradient(int n, const float* in3, float4* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_float4(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2], 0.f);
}
__global__ void scatterSlots(int n, const float* src, const int* slot, float* dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[slot[i]] = src[i];
}
__global__ void scatterRows9(int n, const float* src, const int* slot, float* dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 9; k++) dst[(size_t)9 * slot[i] + k] = src[(size_t)9 * i + k];
}

}  // namespace gbt
