// Persistent frame kernels of the XPBD tissue step.
//
// One launch advances one outer frame: every substep's predict, the graph-coloured Gauss-Seidel
// sweeps (lattice edges, bends, tets), capsule contact, velocity update and the blade's ribbon
// tick (the reference issues ~40 launches per substep for this, V/xpbd/xpbd_solver.cu:3460-3721 and
// V/physics.cu:331-394).  Colours are separated by a barrier instead of a kernel boundary:
//   FrameSync::Grid   cooperative launch over the whole GPU, software grid barrier (bounded spin)
//   FrameSync::Block  one CTA per mesh, __syncthreads (small meshes; the batched instance table)
// Work inside a colour is strided over the participating threads; per-node phases use the same
// node-to-thread map in every phase, so a node's contact, velocity update and next predict need
// no barrier between them.
#include "tissue_device.cuh"
#include "frame_kernels.h"

namespace gbt {

// ---------------------------------------------------------------------------------------------
// barriers
// ---------------------------------------------------------------------------------------------
// Grid barrier on a monotonically increasing arrival counter (reset by the host before launch).
// The arriving thread releases its block's writes with a gpu-scope fence, spins with a clock
// budget, and acquires.  A barrier that times out records kSyncTimeout in the status word; every
// block leaves at its next barrier, so the launch ends and the host reports the error.
constexpr unsigned kSyncTimeout = 1u;

struct GridSync {
    unsigned* counter; unsigned* status; unsigned nblocks; unsigned target;
    long long budget;     // spin budget in SM clock cycles
    unsigned extra;       // arrivals awaited beyond the grid (non-zero only in the timeout test mode)
    __device__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ int size() const { return gridDim.x * blockDim.x; }
    __device__ bool sync() {
        __shared__ unsigned ok;
        __syncthreads();
        target += nblocks;
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(counter, 1u);
            long long start = clock64();
            while (true) {
                unsigned now;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(now) : "l"(counter) : "memory");
                if ((int)(now - (target + extra)) >= 0) break;
                if (*(volatile unsigned*)status != 0u) break;
                if (clock64() - start > budget) { atomicOr(status, kSyncTimeout); break; }
            }
            __threadfence();
            ok = *(volatile unsigned*)status == 0u;
        }
        __syncthreads();
        return ok != 0u;
    }
};

struct BlockSync {
    unsigned* status;
    __device__ int rank() const { return threadIdx.x; }
    __device__ int size() const { return blockDim.x; }
    __device__ bool sync() { __syncthreads(); return true; }
};

// ---------------------------------------------------------------------------------------------
// contact model 0: shaft capsule + jaw slab CCD gate, k_SolveCCDContact (xpbd_solver.cu:1049-1123)
// ---------------------------------------------------------------------------------------------
struct ContactFrame { f3 sa, sb, hinge, axis, normal, w; float shaftR, jawLen, halfWidth, gapHalf, alpha; };

__device__ __forceinline__ f3 lerpTool(float ax, float ay, float az, float bx, float by, float bz, float t) {
    return mk(ax, ay, az) * (1.f - t) + mk(bx, by, bz) * t;
}

// Substep pose of the instrument: linear interpolation from the previous frame's command, then the
// jaw frame orthonormalised (xpbd_solver.cu:3467-3483, 3573-3580).
__device__ __forceinline__ ContactFrame contactFrame(const ToolPose& a, const ToolPose& b, float t, const ContactParams& cp, float alpha) {
    ContactFrame f;
    f.sa = lerpTool(a.sax, a.say, a.saz, b.sax, b.say, b.saz, t);
    f.sb = lerpTool(a.sbx, a.sby, a.sbz, b.sbx, b.sby, b.sbz, t);
    f.hinge = lerpTool(a.hx, a.hy, a.hz, b.hx, b.hy, b.hz, t);
    f3 ax = lerpTool(a.ax, a.ay, a.az, b.ax, b.ay, b.az, t);
    f3 nm = lerpTool(a.nx, a.ny, a.nz, b.nx, b.ny, b.nz, t);
    float gap = a.gap * (1.f - t) + b.gap * t;
    f.axis = len(ax) > 1e-9f ? ax * (1.f / len(ax)) : mk(0.f, 0.f, 1.f);
    f3 n = len(nm) > 1e-9f ? nm * (1.f / len(nm)) : mk(0.f, 1.f, 0.f);
    n = n - f.axis * dot(n, f.axis);
    if (len(n) < 1e-7f) n = cross(f.axis, fabsf(f.axis.x) < 0.9f ? mk(1.f, 0.f, 0.f) : mk(0.f, 1.f, 0.f));
    f.normal = n * (1.f / len(n));
    f.w = cross(f.axis, f.normal);
    f.shaftR = b.shaftR; f.jawLen = b.len; f.halfWidth = b.halfWidth;
    f.gapHalf = 0.5f * fmaxf(gap, cp.jawGapClosed);
    f.alpha = alpha;
    return f;
}

__device__ __forceinline__ void contactNode(const DeviceMesh& m, int c, const ContactFrame& f, const ContactParams& cp) {
    float4 P = m.pos[c];
    float wc = P.w;
    if (wc <= 0.f) return;
    f3 p = xyz(P);
    f3 v = xyz(m.vel[c]);
    {
        f3 ab = f.sb - f.sa;
        float ab2 = dot(ab, ab);
        float tt = ab2 > 1e-12f ? dot(p - f.sa, ab) / ab2 : 0.f;
        tt = fmaxf(0.f, fminf(1.f, tt));
        f3 dv = p - (f.sa + ab * tt);
        float dist = len(dv), C = dist - f.shaftR;
        if (C < 0.f) {
            f3 n = dist > 1e-9f ? dv * (1.f / dist) : mk(0.f, 1.f, 0.f);
            if (-dot(v, n) > cp.ccdVelThresh) {
                float dl = (-C - f.alpha * 0.f) / (wc + f.alpha);
                float ap = cp.ccdOmega * dl;
                f3 corr = n * (wc * ap);
                float cl = len(corr);
                if (cl > cp.ccdMaxDisp) { float s = cp.ccdMaxDisp / cl; ap *= s; corr = corr * s; }
                p = p + corr;
            }
        }
    }
    {
        f3 rel = p - f.hinge;
        float u = dot(rel, f.axis), vv = dot(rel, f.w), n = dot(rel, f.normal);
        if (u >= 0.f && u <= f.jawLen && fabsf(vv) <= f.halfWidth) {
            float an = fabsf(n);
            if (an > f.gapHalf) {
                float C = f.gapHalf - an, sg = n >= 0.f ? 1.f : -1.f;
                f3 nOut = f.normal * sg;
                if (-dot(v, nOut) > cp.ccdVelThresh) {
                    float dl = (-C - f.alpha * 0.f) / (wc + f.alpha);
                    float ap = cp.ccdOmega * dl, cm = wc * ap;
                    if (fabsf(cm) > cp.ccdMaxDisp) { float s = cp.ccdMaxDisp / fabsf(cm); ap *= s; cm *= s; }
                    p = p - f.normal * (sg * cm);
                }
            }
        }
    }
    m.pos[c] = make_float4(p.x, p.y, p.z, wc);
}

// ---------------------------------------------------------------------------------------------
// blade ribbon tick on one lattice edge: CCD crossing, tear law, sever (V/cut.cu:486-746)
// ---------------------------------------------------------------------------------------------
__constant__ int kStencilOff[3][4][3] = {{{0, 0, 0}, {0, -1, 0}, {0, -1, -1}, {0, 0, -1}},
                                         {{0, 0, 0}, {0, 0, -1}, {-1, 0, -1}, {-1, 0, 0}},
                                         {{0, 0, 0}, {-1, 0, 0}, {-1, -1, 0}, {0, -1, 0}}};
__constant__ int kStencilEdge[3][4] = {{0, 2, 6, 4}, {3, 7, 5, 1}, {8, 9, 10, 11}};

__device__ __forceinline__ int nodeId(const DeviceMesh& m, int x, int y, int z) { return x + (m.dx + 1) * (y + (m.dy + 1) * z); }
__device__ __forceinline__ bool voxIn(const DeviceMesh& m, int x, int y, int z) {
    return x >= 0 && y >= 0 && z >= 0 && x < m.dx && y < m.dy && z < m.dz;
}
__device__ __forceinline__ int directedSlot(const DeviceMesh& m, int a, int b) {
    int d = b - a, ad = d < 0 ? -d : d;
    int axis = ad == 1 ? 0 : (ad == m.dx + 1 ? 1 : 2);
    return 6 * a + 2 * axis + (d > 0 ? 1 : 0);
}
__device__ bool edgeIsCut(const DeviceMesh& m, const CutParams& cu, int4 g) {
    for (int s = 0; s < 4; s++) {
        int x = g.y + kStencilOff[g.x][s][0], y = g.z + kStencilOff[g.x][s][1], z = g.w + kStencilOff[g.x][s][2];
        if (voxIn(m, x, y, z) && ((cu.cutMask[x + m.dx * (y + m.dy * z)] >> kStencilEdge[g.x][s]) & 1u)) return true;
    }
    return false;
}
__device__ bool cutHitsMaterial(float t, float skin, int ia, int ib) {
    if (ia && ib) return true;
    if (!ia && !ib) return false;
    if (!(skin >= 0.f && skin <= 1.f)) return false;
    return ia ? t <= skin : t >= skin;
}
// MarkAndEmit (V/cut.cu:218-254): mark the edge in its occupied stencil voxels; on its first cut
// record the fractions and count the two cut-point records of a crossing inside the material.
__device__ void markEdge(const DeviceMesh& m, const CutParams& cu, int4 g, int a, int b, float t) {
    bool first = false, saw = false, occ = false;
    for (int s = 0; s < 4; s++) {
        int x = g.y + kStencilOff[g.x][s][0], y = g.z + kStencilOff[g.x][s][1], z = g.w + kStencilOff[g.x][s][2];
        if (!voxIn(m, x, y, z)) continue;
        int v = x + m.dx * (y + m.dy * z);
        if (cu.occupied[v] == 0u) continue;
        occ = true;
        unsigned bit = 1u << kStencilEdge[g.x][s];
        unsigned old = atomicOr(cu.cutMask + v, bit);
        if (!saw) { saw = true; first = (old & bit) == 0u; }
    }
    if (!(first && occ)) return;
    cu.edgeCutT[directedSlot(m, a, b)] = t;
    cu.edgeCutT[directedSlot(m, b, a)] = 1.f - t;
    if (!cutHitsMaterial(t, cu.skinT[directedSlot(m, a, b)], cu.inside[a], cu.inside[b])) return;
    atomicAdd(cu.counters + 1, 2u);
}

__device__ void tickEdge(const DeviceMesh& m, const CutParams& cu, int e, bool ccd) {
    int4 g = cu.gridEdges[e];          // (axis, x, y, z)
    int axis = g.x;
    int a = nodeId(m, g.y, g.z, g.w);
    int b = nodeId(m, g.y + (axis == 0), g.z + (axis == 1), g.w + (axis == 2));
    int slotA = 6 * a + 2 * axis + 1;
    if (ccd && m.nbr[slotA] >= 0) {
        f3 S = mk(cu.sx, cu.sy, cu.sz), E = mk(cu.ex, cu.ey, cu.ez);
        f3 a0 = xyz(m.prev[a]), a1 = xyz(m.pos[a]), b0 = xyz(m.prev[b]), b1 = xyz(m.pos[b]);
        float pad = cu.voxelL;
        f3 sMin = mk(fminf(S.x, E.x) - pad, fminf(S.y, E.y) - pad, fminf(S.z, E.z) - pad);
        f3 sMax = mk(fmaxf(S.x, E.x) + pad, fmaxf(S.y, E.y) + pad, fmaxf(S.z, E.z) + pad);
        f3 eMin = mk(fminf(fminf(a0.x, a1.x), fminf(b0.x, b1.x)), fminf(fminf(a0.y, a1.y), fminf(b0.y, b1.y)),
                     fminf(fminf(a0.z, a1.z), fminf(b0.z, b1.z)));
        f3 eMax = mk(fmaxf(fmaxf(a0.x, a1.x), fmaxf(b0.x, b1.x)), fmaxf(fmaxf(a0.y, a1.y), fmaxf(b0.y, b1.y)),
                     fmaxf(fmaxf(a0.z, a1.z), fmaxf(b0.z, b1.z)));
        bool cull = eMax.x < sMin.x || eMin.x > sMax.x || eMax.y < sMin.y || eMin.y > sMax.y || eMax.z < sMin.z || eMin.z > sMax.z;
        if (!cull) {
            f3 D = E - S, P0 = a0 - S, Pv = a1 - a0, Q0 = b0 - S, Qv = b1 - b0;
            float c0 = dot(cross(P0, Q0), D), c1 = dot(cross(P0, Qv) + cross(Pv, Q0), D), c2 = dot(cross(Pv, Qv), D);
            float roots[2]; int nr = 0;
            if (fabsf(c2) < 1e-14f) {
                if (fabsf(c1) > 1e-14f) { float r = -c0 / c1; if (r >= 0.f && r <= 1.f) roots[nr++] = r; }
            } else {
                float disc = c1 * c1 - 4.f * c2 * c0;
                if (disc >= 0.f) {
                    float sq = sqrtf(disc), qq = -0.5f * (c1 + (c1 >= 0.f ? sq : -sq));
                    float r0 = qq / c2, r1 = fabsf(qq) > 1e-20f ? c0 / qq : r0;
                    if (r0 > r1) { float tmp = r0; r0 = r1; r1 = tmp; }
                    if (r0 >= 0.f && r0 <= 1.f) roots[nr++] = r0;
                    if (r1 >= 0.f && r1 <= 1.f && r1 != r0) roots[nr++] = r1;
                }
            }
            for (int ri = 0; ri < nr; ri++) {
                float tc = roots[ri];
                f3 pa = a0 + Pv * tc, pb = b0 + Qv * tc, e1 = pb - pa, n2 = cross(e1, D);
                float n2l = dot(n2, n2);
                if (n2l < 1e-16f) continue;
                f3 wv = S - pa;
                float u = dot(cross(wv, D), n2) / n2l, v = dot(cross(wv, e1), n2) / n2l;
                if (u <= 0.f || u > 1.f || v < -2e-2f || v > 1.f + 2e-2f) continue;
                markEdge(m, cu, g, a, b, u);
                break;
            }
        }
    }
    if (cu.tearLen2 > 0.f && m.nbr[slotA] >= 0 && m.active[a] != 0 && m.active[b] != 0 && !edgeIsCut(m, cu, g)) {
        bool anyOcc = false;
        for (int s = 0; s < 4 && !anyOcc; s++) {
            int x = g.y + kStencilOff[axis][s][0], y = g.z + kStencilOff[axis][s][1], z = g.w + kStencilOff[axis][s][2];
            anyOcc = voxIn(m, x, y, z) && cu.occupied[x + m.dx * (y + m.dy * z)] != 0u;
        }
        if (anyOcc) {
            f3 d = xyz(m.pos[b]) - xyz(m.pos[a]);
            float l2 = dot(d, d);
            f3 r = xyz(cu.rest[b]) - xyz(cu.rest[a]);
            float tl2 = cu.tearLen2 * (dot(r, r) / (cu.voxelL * cu.voxelL));
            if (l2 > tl2) {
                atomicAdd(cu.counters + 2, 1u);
                markEdge(m, cu, g, a, b, 0.5f);
            }
        }
    }
    // SeverLinks (V/cut.cu:719-746): a cut mark on this edge parts the link and its bend pairs.
    bool valid = true;
    for (int s = 0; s < 4; s++)
        valid = valid && voxIn(m, g.y + kStencilOff[axis][s][0], g.z + kStencilOff[axis][s][1], g.w + kStencilOff[axis][s][2]);
    if (!valid || !edgeIsCut(m, cu, g)) return;
    if (m.nbr[slotA] >= 0) atomicAdd(cu.counters + 0, 1u);
    m.nbr[slotA] = -1;
    m.nbr[6 * b + 2 * axis] = -1;
    if (m.nBendPairs >= 15 * (max(a, b) + 1)) {
        for (int p = 0; p < 15; p++) {
            BendRecord* x = m.bendPairs + 15 * a + p;
            if (x->alive != 0 && (x->j == b || x->k == b)) x->alive = 0;
            BendRecord* y = m.bendPairs + 15 * b + p;
            if (y->alive != 0 && (y->j == a || y->k == a)) y->alive = 0;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// frame driver
// ---------------------------------------------------------------------------------------------
template <class Sync>
__device__ void runFrame(const DeviceMesh& m, const FrameCoeffs& fc, const ToolPose& from, const ToolPose& to,
                         const ContactParams& cp, const CutParams& cu, unsigned* state, Sync& sync) {
    const int r = sync.rank(), R = sync.size();
    // state[0]: topology revision the liveness flags were derived at (~0u: never)
    unsigned derivedAt = *(volatile unsigned*)state;
    bool havePrev = cu.havePrev != 0;
    for (int s = 0; s < fc.substeps; s++) {
        // -- liveness refresh when the topology moved (k_TopologyStale + k_RefreshLiveness) --
        unsigned revision = cu.counters ? *(volatile unsigned*)(cu.counters) : 0u;
        bool stale = derivedAt != revision || derivedAt == ~0u;
        if (stale) {
            if (fc.fallback) {
                for (int i = r; i < 6 * m.nNodes; i += R) m.edgeSupport[i] = 0;
                if (!sync.sync()) return;
            }
            for (int e = r; e < m.nEdges; e += R) refreshEdge(m, e);
            for (int b = r; b < m.nBends; b += R) m.bendLive[b] = m.bendPairs[m.bendSrc[b]].alive != 0 ? 1 : 0;
            for (int k = r; k < m.nTets; k += R) {
                refreshTet(m, k);
                if (fc.fallback && (m.tetMeta[k] & 8))
                    for (int o = 0; o < 3; o++) m.edgeSupport[m.tetOwner[3 * k + o]] = 1;
            }
            derivedAt = revision;
        }
        // -- predict (k_predict) --
        for (int i = r; i < m.nNodes; i += R) {
            float4 P = m.pos[i];
            if (stale) P.w = nodeInvMass(m, i);
            m.prev[i] = make_float4(P.x, P.y, P.z, 0.f);
            if (P.w > 0.f) {
                float4 F = m.ext[i], V = m.vel[i];
                f3 a = mk(F.x, F.y, F.z) * P.w;
                f3 v = xyz(V) + a * fc.h;
                m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
                f3 x = xyz(P) + v * fc.h;
                P = make_float4(x.x, x.y, x.z, P.w);
            }
            m.pos[i] = P;
        }
        if (!sync.sync()) return;
        // -- coloured Gauss-Seidel sweeps --
        if (fc.doEdges)
            for (int c = 0; c < m.nEdgeColors; c++) {
                int lo = m.edgeColorOff[c], hi = m.edgeColorOff[c + 1];
                for (int e = lo + r; e < hi; e += R) projectEdge(m, e, fc);
                if (!sync.sync()) return;
            }
        if (fc.doBend)
            for (int c = 0; c < m.nBendColors; c++) {
                int lo = m.bendColorOff[c], hi = m.bendColorOff[c + 1];
                for (int e = lo + r; e < hi; e += R) projectBend(m, e, fc);
                if (!sync.sync()) return;
            }
        if (fc.doStrain)
            for (int c = 0; c < m.nTetColors; c++) {
                int lo = m.tetColorOff[c], hi = m.tetColorOff[c + 1];
                for (int k = lo + r; k < hi; k += R) projectTet(m, k, fc);
                if (!sync.sync()) return;
            }
        // -- contact, velocity --
        float t = fminf(1.f, (float)(fc.firstSubstep + s + 1) / (float)fc.numSubsteps);
        ContactFrame cf;
        if (fc.contact) cf = contactFrame(from, to, t, cp, fc.contactAlphaH2);
        for (int i = r; i < m.nNodes; i += R) {
            if (fc.contact) contactNode(m, i, cf, cp);
            float4 P = m.pos[i], Q = m.prev[i];
            f3 v = P.w > 0.f ? (xyz(P) - xyz(Q)) * fc.invH : mk(0.f, 0.f, 0.f);
            if (!fc.perpDamp) v = P.w > 0.f ? v * fc.velScale : mk(0.f, 0.f, 0.f);
            m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
        }
        if (fc.perpDamp) {   // k_perp_damp_edges between the raw velocity write and the Rayleigh scale
            if (!sync.sync()) return;
            for (int c = 0; c < m.nEdgeColors; c++) {
                int lo = m.edgeColorOff[c], hi = m.edgeColorOff[c + 1];
                for (int e = lo + r; e < hi; e += R) {
                    if (m.edgeLive[e] == 0) continue;
                    int2 ij = m.edgeEnds[e];
                    float4 Pi = m.pos[ij.x], Pj = m.pos[ij.y];
                    float wi = Pi.w, wj = Pj.w;
                    if (wi + wj <= 0.f) continue;
                    f3 d = xyz(Pi) - xyz(Pj);
                    float L = len(d);
                    if (L < 1e-9f) continue;
                    f3 n = d * (1.f / L), vi = xyz(m.vel[ij.x]), vj = xyz(m.vel[ij.y]), vr = vi - vj;
                    f3 imp = (vr - n * dot(vr, n)) * (fc.h * fc.betaS);
                    if (wi > 0.f) { vi = vi - imp * wi; m.vel[ij.x] = make_float4(vi.x, vi.y, vi.z, 0.f); }
                    if (wj > 0.f) { vj = vj + imp * wj; m.vel[ij.y] = make_float4(vj.x, vj.y, vj.z, 0.f); }
                }
                if (!sync.sync()) return;
            }
            for (int i = r; i < m.nNodes; i += R) {
                float4 V = m.vel[i];
                f3 v = m.pos[i].w > 0.f ? xyz(V) * fc.velScale : mk(0.f, 0.f, 0.f);
                m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
            }
        }
        // -- blade ribbon tick between substeps --
        if (fc.cut) {   // the first tick after the blade is set only takes the position snapshot
            if (havePrev) {
                if (!sync.sync()) return;
                for (int e = r; e < cu.nGridEdges; e += R) tickEdge(m, cu, e, true);
                if (!sync.sync()) return;
            }
            havePrev = true;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *(volatile unsigned*)state = derivedAt;
}

__global__ void __launch_bounds__(kFrameThreads) frameKernelGrid(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                  ContactParams cp, CutParams cu, unsigned* state) {
    GridSync g{state + 1, state + 2, gridDim.x, 0u, fc.spinBudget, (unsigned)fc.syncTestExtra};
    runFrame(m, fc, from, to, cp, cu, state, g);
}

__global__ void __launch_bounds__(kFrameThreads) frameKernelBlock(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                   ContactParams cp, CutParams cu, unsigned* state) {
    BlockSync b{state + 2};
    runFrame(m, fc, from, to, cp, cu, state, b);
}

// Per-tet compliance of the frame, k_ComputeTetAlpha (xpbd_solver.cu:578-587).
__global__ void tetAlphaKernel(int n, float invH2, const float2* stiff, float2* alpha) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) { float2 s = stiff[k]; alpha[k] = make_float2(invH2 / s.x, invH2 / s.y); }
}

// Body force = acceleration * mass, k_SetGravity (V/physics.cu:317-321).  ext.w holds the mass.
__global__ void gravityKernel(int n, float gx, float gy, float gz, float4* ext) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { float mass = ext[i].w; ext[i] = make_float4(gx * mass, gy * mass, gz * mass, mass); }
}

// Rod-phase blade detection, k_DetectCutQuad + k_SeverLinks (V/cut.cu:421-474, 719-746): the swept quad's
// two triangles against every deformed lattice edge.


__device__ bool mollerTrumbore(f3 O, f3 D, f3 V0, f3 V1, f3 V2, float& t) {
    f3 L1 = V1 - V0, L2 = V2 - V0, T = V0 - O;
    float det = dot(cross(L2, D), L1);
    t = 0.f;
    if (fabsf(det) < 1e-12f) return false;
    float inv = 1.f / det;
    t = dot(cross(L2, T), L1) * inv;
    float u = -dot(cross(L2, D), T) * inv;
    float v = dot(cross(D, T), L1) * inv;
    const float EPS = 1e-5f;
    return u >= -EPS && v >= -EPS && u + v <= 1.f + EPS && t > 0.f && t <= 1.f;
}

__global__ void detectQuadKernel(DeviceMesh m, CutParams cu, QuadTool tool) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cu.nGridEdges || !tool.valid) return;
    int4 g = cu.gridEdges[e];
    int axis = g.x;
    int a = nodeId(m, g.y, g.z, g.w), b = nodeId(m, g.y + (axis == 0), g.z + (axis == 1), g.w + (axis == 2));
    f3 O = xyz(m.pos[a]), D = xyz(m.pos[b]) - O;
    float pad = cu.voxelL;
    f3 mn = mk(fminf(O.x, O.x + D.x), fminf(O.y, O.y + D.y), fminf(O.z, O.z + D.z));
    f3 mx = mk(fmaxf(O.x, O.x + D.x), fmaxf(O.y, O.y + D.y), fmaxf(O.z, O.z + D.z));
    if (mx.x < tool.lo.x - pad || mn.x > tool.hi.x + pad || mx.y < tool.lo.y - pad || mn.y > tool.hi.y + pad ||
        mx.z < tool.lo.z - pad || mn.z > tool.hi.z + pad) return;
    float t1, t2;
    bool h1 = mollerTrumbore(O, D, tool.t1[0], tool.t1[1], tool.t1[2], t1);
    bool h2 = mollerTrumbore(O, D, tool.t2[0], tool.t2[1], tool.t2[2], t2);
    if (!h1 && !h2) return;
    float tr = (h1 && h2) ? fminf(t1, t2) : (h1 ? t1 : t2);
    tr = fminf(fmaxf(tr, 0.f), 1.f);
    markEdge(m, cu, g, a, b, tr);
}

__global__ void severKernel(DeviceMesh m, CutParams cu) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cu.nGridEdges) return;
    CutParams noTear = cu;
    noTear.tearLen2 = 0.f;
    tickEdge(m, noTear, e, false);
}

}  // namespace gbt
