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
#include <cooperative_groups.h>

#include "tissue_device.cuh"
#include "grid_sync.cuh"
#include "friction_contact.cuh"
#include "particle_frame.cuh"
#include "frame_kernels.h"

namespace gbt {

// ---------------------------------------------------------------------------------------------
// contact model 0: shaft capsule + jaw slab CCD gate, k_SolveCCDContact (xpbd_solver.cu:1049-1123)
// ---------------------------------------------------------------------------------------------
// The substep's instrument frame (contactFrame) lives in tissue_device.cuh: batches evaluate it on
// the host, single meshes on the device, with the same operations.
// The contact of one mobile node (wc > 0) at p moving with the substep's predicted velocity v.
// Warp-level early-out of the capsule test: a node outside the box of the shaft segment grown by the
// radius (and a margin far above the rounding of the exact distance) cannot be inside the capsule,
// where the exact test would change nothing; a warp with no node inside that box skips the test
// (one ballot), the others run it exactly as before, so the result is the same bit for bit.
__device__ __forceinline__ bool nearCapsule(f3 p, const ContactFrame& f) {
    const float r = f.shaftR * 1.0001f + 1e-5f;
    return p.x >= fminf(f.sa.x, f.sb.x) - r && p.x <= fmaxf(f.sa.x, f.sb.x) + r && p.y >= fminf(f.sa.y, f.sb.y) - r &&
           p.y <= fmaxf(f.sa.y, f.sb.y) + r && p.z >= fminf(f.sa.z, f.sb.z) - r && p.z <= fmaxf(f.sa.z, f.sb.z) + r;
}
__device__ __forceinline__ f3 contactPoint(f3 p, float wc, f3 v, const ContactFrame& f, const ContactParams& cp) {
    const bool near = nearCapsule(p, f);
    if (__ballot_sync(__activemask(), near) != 0u && near) {
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
    return p;
}
template <bool Dsm = false>
__device__ __forceinline__ void contactNode(const DeviceMesh& m, int c, const ContactFrame& f, const ContactParams& cp) {
    const float4 P = posRef<Dsm>(m, c);
    if (P.w <= 0.f) return;
    const f3 p = contactPoint(xyz(P), P.w, xyz(m.vel[c]), f, cp);
    posRef<Dsm>(m, c) = make_float4(p.x, p.y, p.z, P.w);
}

// k_predict on one node whose position P (w = inverse mass), velocity V and external force F are
// in registers: x_prev = x; v += h f w; x += h v.
template <bool Dsm = false>
__device__ __forceinline__ float4 predictNode(const DeviceMesh& m, int i, float4 P, f3 V, float4 F, float h) {
    m.prev[i] = make_float4(P.x, P.y, P.z, 0.f);
    if (P.w > 0.f) {
        f3 a = mk(F.x, F.y, F.z) * P.w;
        f3 v = V + a * h;
        m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
        f3 x = xyz(P) + v * h;
        P = make_float4(x.x, x.y, x.z, P.w);
    }
    posRef<Dsm>(m, i) = P;
    return P;
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
// EmitCutPoint (V/cut.cu:186-215): the cut point of owner p on the undeformed edge (`along`) plus
// the half-kerf on p's side of the cut plane, and the outward cut normal, both in p's frame `rot`.
__device__ void emitCutPoint(const DeviceMesh& m, const CutParams& cu, const float* rot, f3 hit, f3 along, int p, int slot, f3 ncut) {
    const f3 pp = xyz(m.pos[p]);
    const float sd = dot(pp - hit, ncut);
    float side = sd > 0.f ? 1.f : (sd < 0.f ? -1.f : 0.f);
    if (side == 0.f) side = 1.f;
    const float* q = rot + 9 * (size_t)p;
    const f3 r0 = mk(q[0], q[1], q[2]), r1 = mk(q[3], q[4], q[5]), r2 = mk(q[6], q[7], q[8]);
    const f3 g = ncut * (side * (cu.toolD * 0.5f)), n = ncut * side;
    const f3 local = along + ((r0 * g.x + r1 * g.y) + r2 * g.z);
    const f3 mat = (r0 * n.x + r1 * n.y) + r2 * n.z;
    cu.cutRec[2 * (size_t)slot] = make_float4(local.x, local.y, local.z, 1.f);
    cu.cutRec[2 * (size_t)slot + 1] = make_float4(mat.x, mat.y, mat.z, 0.f);
}

// MarkAndEmit (V/cut.cu:218-254): mark the edge in its occupied stencil voxels; on its first cut
// record the fractions and, for a crossing inside the material, the two cut points (the owners'
// frames `rot`; `hit` and `ncut` place the kerf).
__device__ void markEdge(const DeviceMesh& m, const CutParams& cu, const float* rot, int4 g, int a, int b, float t, f3 hit, f3 ncut) {
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
    if (cu.cutRec && rot) {
        const f3 rest = xyz(cu.rest[b]) - xyz(cu.rest[a]);
        emitCutPoint(m, cu, rot, hit, rest * t, a, 6 * a + 2 * g.x + 1, ncut);
        emitCutPoint(m, cu, rot, hit, rest * (t - 1.f), b, 6 * b + 2 * g.x, ncut);
    }
}

__device__ void tickEdgeAt(const DeviceMesh& m, const CutParams& cu, int4 g, bool ccd, const float* rot) {
    int axis = g.x;                    // g = (axis, x, y, z) of the base node
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
                // hit on the current edge; kerf normal = blade x relative tissue motion, else the
                // last valid blade normal (V/cut.cu:576-587)
                const f3 hit = a1 + (b1 - a1) * u;
                const f3 relV = (Pv + Qv) * 0.5f, nHit = cross(D, relV);
                const float nLen = len(nHit);
                const f3 nEmit = nLen > 1e-8f ? mk(nHit.x / nLen, nHit.y / nLen, nHit.z / nLen) : mk(cu.ncx, cu.ncy, cu.ncz);
                markEdge(m, cu, rot, g, a, b, u, hit, nEmit);
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
            if (l2 > tl2) {   // tear plane normal to the edge through its midpoint (V/cut.cu:674-683)
                atomicAdd(cu.counters + 2, 1u);
                const float l = sqrtf(l2);
                markEdge(m, cu, rot, g, a, b, 0.5f, xyz(m.pos[a]) + d * 0.5f, mk(d.x / l, d.y / l, d.z / l));
            }
        }
    }
    // SeverLinks (V/cut.cu:719-746): a cut mark on this edge parts the link and its bend pairs.
    bool valid = true;
    for (int s = 0; s < 4; s++)
        valid = valid && voxIn(m, g.y + kStencilOff[axis][s][0], g.z + kStencilOff[axis][s][1], g.w + kStencilOff[axis][s][2]);
    if (!valid || !edgeIsCut(m, cu, g)) return;
    // When every live bend pair's links exist (checked when the physics is set up, and kept: a
    // sever kills the pairs of the link it removes), an edge whose link is already gone has no live
    // pair left, and the pass below would change nothing.
    if (cu.skipSevered && m.nbr[slotA] < 0) return;
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
// tissue guard: the feasibility chain after contact (finishFeasible, xpbd_solver.cu:628-741)
__device__ __forceinline__ void tickEdge(const DeviceMesh& m, const CutParams& cu, int e, bool ccd, const float* rot) {
    tickEdgeAt(m, cu, cu.gridEdges[e], ccd, rot);
}

// Brick pre-cull of the ribbon tick: the lattice's base nodes in bricks of 4 x 4 x 4, each brick's
// box over the current and substep-start positions of its nodes and of the +1 layer that its edges
// reach.  An edge whose brick box misses the blade's padded box misses it too, so only the edges of
// listed bricks run the crossing test; the rest of the tick (the sever of marked edges) has nothing
// to do on the others: rod-phase marks are severed when made, tick marks are made on listed edges,
// and the tear law (which visits every edge) keeps the full pass.
constexpr int kBrick = 4, kBrickEdges = 3 * kBrick * kBrick * kBrick;
__device__ void brickBounds(const DeviceMesh& m, const CutParams& cu, int b, int lane) {
    const int nbx = (m.dx + kBrick - 1) / kBrick, nby = (m.dy + kBrick - 1) / kBrick;
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    const int x0 = bx * kBrick, y0 = by * kBrick, z0 = bz * kBrick;
    const int x1 = min(x0 + kBrick, m.dx), y1 = min(y0 + kBrick, m.dy), z1 = min(z0 + kBrick, m.dz);
    // the (kBrick + 1)^3 = 125 node slots of the brick, four per lane (constant divisors), all loads
    // issued before any use; slots past the lattice's last layer are skipped
    constexpr int kSide = kBrick + 1;
    f3 lo = mk(3.0e38f, 3.0e38f, 3.0e38f), hi = mk(-3.0e38f, -3.0e38f, -3.0e38f);
    float4 P[4], Q[4];
    bool in[4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int k = lane + 32 * t;
        const int x = x0 + k % kSide, y = y0 + (k / kSide) % kSide, z = z0 + k / (kSide * kSide);
        in[t] = k < kSide * kSide * kSide && x <= x1 && y <= y1 && z <= z1;
        if (in[t]) { const int id = nodeId(m, x, y, z); P[t] = m.pos[id]; Q[t] = m.prev[id]; }
    }
#pragma unroll
    for (int t = 0; t < 4; t++) {
        if (!in[t]) continue;
        const f3 p = xyz(P[t]), q = xyz(Q[t]);
        lo = mk(fminf(lo.x, fminf(p.x, q.x)), fminf(lo.y, fminf(p.y, q.y)), fminf(lo.z, fminf(p.z, q.z)));
        hi = mk(fmaxf(hi.x, fmaxf(p.x, q.x)), fmaxf(hi.y, fmaxf(p.y, q.y)), fmaxf(hi.z, fmaxf(p.z, q.z)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = mk(fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o)), fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o)),
                fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o)));
        hi = mk(fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o)), fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o)),
                fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o)));
    }
    if (lane != 0) return;
    const float pad = cu.voxelL;
    const bool miss = hi.x < fminf(cu.sx, cu.ex) - pad || lo.x > fmaxf(cu.sx, cu.ex) + pad ||
                      hi.y < fminf(cu.sy, cu.ey) - pad || lo.y > fmaxf(cu.sy, cu.ey) + pad ||
                      hi.z < fminf(cu.sz, cu.ez) - pad || lo.z > fmaxf(cu.sz, cu.ez) + pad;
    if (!miss) {
        const unsigned slot = atomicAdd(cu.brickCount, 1u);
        if (slot < (unsigned)cu.nBricks) cu.brickList[slot] = b;
    }
}
// Edge `l` (0 .. kBrickEdges-1) of a listed brick as (axis, base node), or false when the lattice has
// no such interior edge (one whose four incident voxels exist, as the host's edge list holds).
__device__ __forceinline__ bool brickEdge(const DeviceMesh& m, int b, int l, int4& g) {
    const int nbx = (m.dx + kBrick - 1) / kBrick, nby = (m.dy + kBrick - 1) / kBrick;
    const int axis = l / (kBrick * kBrick * kBrick), o = l % (kBrick * kBrick * kBrick);
    const int x = (b % nbx) * kBrick + o % kBrick, y = ((b / nbx) % nby) * kBrick + (o / kBrick) % kBrick,
              z = (b / (nbx * nby)) * kBrick + o / (kBrick * kBrick);
    const int c[3] = {x, y, z}, d[3] = {m.dx, m.dy, m.dz};
    for (int a = 0; a < 3; a++)
        if (a == axis ? c[a] >= d[a] : (c[a] < 1 || c[a] >= d[a])) return false;
    g = make_int4(axis, x, y, z);
    return true;
}

// ---------------------------------------------------------------------------------------------
// If a live tet is below the minimum relative volume: two colour sweeps of a linearised repair; if
// one still is: every vertex of a tet whose substep motion may pass below the minimum restarts from
// its substep-start position and advances as far as its incident live tets allow, in eight
// lattice-parity colours whose order rotates with the substep index.  The flags are written by any
// thread and read by all after a barrier, so every branch below is uniform.
template <class Sync>
__device__ bool guardFeasible(const DeviceMesh& m, const FrameCoeffs& fc, int substepIndex, Sync& sync) {
    const int r = sync.spreadRank(), R = sync.size();
    const int T = m.nTetColors > 0 ? m.tetRange[m.nTetColors - 1].y : 0;
    const int nodeEnd = m.nodeBase + m.nNodes;
    const float minimum = fc.minVolume;
    if (sync.leader()) { m.guardFlags[0] = 0u; m.guardFlags[1] = 0u; }
    for (int i = m.nodeBase + r; i < nodeEnd; i += R) m.needed[i] = 0;
    if (!sync.sync()) return false;
    for (int k = r; k < T; k += R) {
        int meta = m.tetMeta[k];
        if ((meta & 8) == 0) continue;
        float J = tetVolume(m, k, meta);
        if (!isfinite(J) || J < minimum) m.guardFlags[0] = 1u;
    }
    if (!sync.sync()) return false;
    if (*(volatile unsigned*)&m.guardFlags[0] == 0u) return true;
    for (int pass = 0; pass < 2; pass++)
        for (int c = 0; c < m.nTetColors; c++) {
            int2 rg = m.tetRange[c];
            for (int k = rg.x + r; k < rg.y; k += R) repairTet(m, k, minimum);
            if (!sync.sync()) return false;
        }
    for (int k = r; k < T; k += R) {
        int meta = m.tetMeta[k];
        if ((meta & 8) == 0) continue;
        float J = tetVolume(m, k, meta);
        if (!isfinite(J) || J < minimum) m.guardFlags[1] = 1u;
    }
    if (!sync.sync()) return false;
    if (*(volatile unsigned*)&m.guardFlags[1] == 0u) return true;
    for (int k = r; k < T; k += R) needFeasible(m, k, minimum);
    if (!sync.sync()) return false;
    for (int i = m.nodeBase + r; i < nodeEnd; i += R)
        if (m.needed[i]) {
            float4 P = m.pos[i], Q = m.prev[i];
            m.feasTarget[i] = P;
            m.pos[i] = make_float4(Q.x, Q.y, Q.z, P.w);
        }
    if (!sync.sync()) return false;
    const int nx = m.dx + 1, ny = m.dy + 1, nz = m.dz + 1;
    const int cx = (nx + 1) / 2, cy = (ny + 1) / 2, cz = (nz + 1) / 2, sites = cx * cy * cz;
    for (int k = 0; k < 8; k++) {
        int color = (k + substepIndex) & 7;
        for (int lane = r; lane < sites; lane += R) {
            int x = 2 * (lane % cx) + (color & 1), y = 2 * ((lane / cx) % cy) + ((color >> 1) & 1), z = 2 * (lane / (cx * cy)) + ((color >> 2) & 1);
            if (x >= nx || y >= ny || z >= nz) continue;
            feasibleVertex(m, x + nx * (y + ny * z), minimum);
        }
        if (!sync.sync()) return false;
    }
    return true;
}

// Contact model 1 over this thread's nodes: every node against the shaft capsule and both jaw
// boxes (kept out of line so its shapes do not enlarge the frame kernel's register allocation).
__device__ __noinline__ void frictionPhase(const DeviceMesh& m, const FrameCoeffs& fc, const ToolPose& from, const ToolPose& to,
                                           const ContactParams& cp, float t, int r, int R) {
    const float previousT = fmaxf(0.f, t - 1.f / (float)fc.numSubsteps);
    const FrictionShapes fs = frictionShapes(from, to, t, previousT, fc.jawThickness, cp.jawGapClosed);
    for (int i = m.nodeBase + r; i < m.nodeBase + m.nNodes; i += R) frictionNode(m, i, fs, fc.contactRadius, fc.contactAlphaH2, fc.muS, fc.muD);
}

// ---------------------------------------------------------------------------------------------
// frame driver
// ---------------------------------------------------------------------------------------------
// Extended: the tissue guard and contact model 1 are compiled in.  Kernels without them keep the
// plain path's register allocation (the extended kernel launches only when either is armed).
// Dsm: node positions live in the cluster's distributed shared memory (cluster batch kernel).
// Rotations: the session kernels, which also compute the particle frames (batched instances do not).
// EdgeGroup: a thread takes its edges of a colour this many at a time (2 in the whole-GPU kernels;
// four at a time measured slower on the batch: the extra registers spill).
// Ahead (only where registers allow: the one-CTA-per-SM kernels): with edge pairs, the thread's
// first pair of colour c+1 is loaded before colour c's edges are projected, and the node passes
// take two nodes at a time.
// Codes: batched instances, whose element tables may be the implicit lattice codes.
template <class Sync, bool Extended, bool Dsm = false, bool Rotations = false, int EdgeGroup = 1, bool Ahead = false, bool Codes = false>
__device__ void runFrame(const DeviceMesh& m, const FrameCoeffs& fc, const ToolPose& from, const ToolPose& to,
                         const ContactParams& cp, const CutParams& cu, unsigned* state, Sync& sync) {
    const int r = sync.spreadRank(), R = sync.size();
    const bool guarded = Extended && fc.guarded != 0;
    // state[0]: topology revision the liveness flags were derived at (~0u: never)
    unsigned derivedAt = *(volatile unsigned*)state;
    bool havePrev = cu.havePrev != 0;
    // Section profiler: the first thread of CTA 0 stamps the global timer when each phase ends.
    const bool stamp = fc.phaseClock != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
    int slot = 0;
    auto mark = [&](int s, unsigned tag) {
        if (stamp && slot < kPhaseRecordsPerSubstep) {
            unsigned long long ns;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(ns));
            fc.phaseClock[(size_t)s * kPhaseRecordsPerSubstep + slot++] = ((unsigned long long)tag << 56) | (ns & 0x00FFFFFFFFFFFFFFull);
        }
    };
    // particle frames from the current state into the other buffer (physics_compute_rotations,
    // V/physics.cu:399-411); every thread takes its own nodes, the caller synchronises around it.
    // Session kernels only, where positions are plain memory (Dsm is false).
    const bool rotations = Rotations && fc.rotations != 0;
    int rotParity = fc.rotParity;
    bool predicted = false;   // the substep's predict already ran in the previous substep's velocity pass
    bool edge0Done = false;   // ... and so did its colour-0 edges
    auto framePass = [&]() {
        const float* prevRot = m.particleRot[rotParity];
        float* rot = m.particleRot[rotParity ^ 1];
        for (int i = m.nodeBase + r; i < m.nodeBase + m.nNodes; i += R) particleFrame(i, m.pos, m.nbr, m.active, m.pinned, prevRot, rot);
        rotParity ^= 1;
    };
    for (int s = 0; s < fc.substeps; s++) {
        slot = 0;
        mark(s, kPhaseFrameStart);
        // -- liveness refresh when the topology moved (k_TopologyStale + k_RefreshLiveness) --
        unsigned revision = cu.counters ? *(volatile unsigned*)(cu.counters) : 0u;
        bool stale = derivedAt != revision || derivedAt == ~0u;
        if (stale) {
            if (fc.fallback) {
                for (int i = 6 * m.nodeBase + r; i < 6 * (m.nodeBase + m.nNodes); i += R) m.edgeSupport[i] = 0;
                if (!sync.sync()) return;
            }
            for (int c = 0; c < m.nEdgeColors; c++)
                for (int e = m.edgeRange[c].x + r; e < m.edgeRange[c].y; e += R) refreshEdge<Codes>(m, e);
            for (int c = 0; c < m.nBendColors; c++)
                for (int b = m.bendRange[c].x + r; b < m.bendRange[c].y; b += R) m.bendLive[b] = m.bendPairs[m.bendSrc[b]].alive != 0 ? 1 : 0;
            for (int c = 0; c < m.nTetColors; c++)
                for (int k = m.tetRange[c].x + r; k < m.tetRange[c].y; k += R) {
                    refreshTet<Codes>(m, k);
                    if (fc.fallback && (m.tetMeta[k] & 8))
                        for (int o = 0; o < 3; o++) m.edgeSupport[checkSlot(m, m.tetOwner[3 * k + o], kSiteTetSlot)] = 1;
                }
            derivedAt = revision;
        }
        const int nodeEnd = m.nodeBase + m.nNodes;
        // -- predict (k_predict), unless the previous substep's velocity pass already did it --
        // With Ahead a thread takes its nodes two at a time, both nodes' loads ahead of either's stores.
        // As in the velocity pass below, the ends of each colour-0 edge are predicted by one thread,
        // which projects the edge on the spot (not while the liveness flags are derived again: edge
        // support comes from every tet's refresh, which only the barrier orders before the edge).
        if (!Codes && !Dsm && !Extended && !predicted && !stale && m.fuseEdge0 && fc.doEdges && m.nEdgeColors > 0) {
            FrameCoeffs noStart = fc;
            noStart.betaGammaHS = 0.f;   // the record's substep-start ends come from the registers below
            const int2 g0 = m.edgeRange[0];
            for (int e = g0.x + r; e < g0.y; e += R) {
                EdgeRecord er = loadEdge<false>(m, e, noStart);
                const int a = er.ij.x, b = er.ij.y;
                const float4 Pa = posRef<Dsm>(m, a), Va = m.vel[a], Fa = m.ext[a];
                const float4 Pb = posRef<Dsm>(m, b), Vb = m.vel[b], Fb = m.ext[b];
                er.qi = xyz(Pa);
                er.qj = xyz(Pb);
                const float4 Na = predictNode<Dsm>(m, a, Pa, xyz(Va), Fa, fc.h);
                const float4 Nb = predictNode<Dsm>(m, b, Pb, xyz(Vb), Fb, fc.h);
                float4 oa, ob;
                if (solveEdge(er, fc, Na, Nb, oa, ob)) {
                    posRef<Dsm>(m, a) = oa;
                    posRef<Dsm>(m, b) = ob;
                }
            }
            for (int q = r; q < m.nUncovered0; q += R) {
                const int i = m.uncovered0[q];
                const float4 Pi = posRef<Dsm>(m, i), Vi = m.vel[i], Fi = m.ext[i];
                predictNode<Dsm>(m, i, Pi, xyz(Vi), Fi, fc.h);
            }
            edge0Done = true;
        } else if (!predicted && Codes && m.mobile) {
            for (int q = r; q < m.nMobile; q += R) {
                const int i = m.mobile[q];
                float4 Pi = posRef<Dsm>(m, i);
                const float4 Vi = m.vel[i], Fi = m.ext[i];
                if (stale) Pi.w = nodeInvMass(m, i);
                predictNode<Dsm>(m, i, Pi, xyz(Vi), Fi, fc.h);
            }
        } else if (!predicted)
            for (int i = m.nodeBase + r; i < nodeEnd; i += (Ahead ? 2 : 1) * R) {
                const int j = Ahead ? i + R : nodeEnd;
                float4 Pi = posRef<Dsm>(m, i), Vi = m.vel[i], Fi = m.ext[i], Pj, Vj, Fj;
                if (j < nodeEnd) { Pj = posRef<Dsm>(m, j); Vj = m.vel[j]; Fj = m.ext[j]; }
                if (stale) Pi.w = nodeInvMass(m, i);
                predictNode<Dsm>(m, i, Pi, xyz(Vi), Fi, fc.h);
                if (j < nodeEnd) {
                    if (stale) Pj.w = nodeInvMass(m, j);
                    predictNode<Dsm>(m, j, Pj, xyz(Vj), Fj, fc.h);
                }
            }
        predicted = false;
        if (!sync.sync()) return;
        mark(s, kPhasePredict);
        // -- coloured Gauss-Seidel sweeps --
        // Tets: a thread loads the record of its first tet of colour c+1 (indices, rest data and
        // substep-start positions, none of which the sweep writes) before the barrier that closes
        // colour c, so only the gathers of current positions follow the barrier.  (Loading further
        // ahead inside a colour costs more in registers, hence occupancy, than it saves; measured.)
        // the thread's first tet of colour 0 (loaded before the last edge barrier with Ahead)
        TetRecord next;
        bool hasNext = false, tetLoaded = false;
        auto loadFirstTet = [&]() {
            const int2 first = m.nTetColors > 0 ? m.tetRange[0] : make_int2(0, 0);
            hasNext = first.x + r < first.y;
            if (hasNext) next = loadTet<Codes>(m, first.x + r, fc);
            tetLoaded = true;
        };
        const int firstEdgeColour = edge0Done ? 1 : 0;
        edge0Done = false;
        if (fc.doEdges) {
            EdgeRecord n0, n1;
            bool h0 = false, h1 = false;
            if (Ahead && EdgeGroup == 2 && m.nEdgeColors > firstEdgeColour) {
                const int2 g0 = m.edgeRange[firstEdgeColour];
                h0 = g0.x + r < g0.y; h1 = g0.x + r + R < g0.y;
                if (h0) n0 = loadEdge<Codes>(m, g0.x + r, fc);
                if (h1) n1 = loadEdge<Codes>(m, g0.x + r + R, fc);
            }
            for (int c = firstEdgeColour; c < m.nEdgeColors; c++) {
                int2 rg = m.edgeRange[c];
                if (Ahead && EdgeGroup == 2) {
                    const EdgeRecord c0 = n0, c1 = n1;
                    const bool k0 = h0, k1 = h1;
                    if (c + 1 < m.nEdgeColors) {
                        const int2 ng = m.edgeRange[c + 1];
                        h0 = ng.x + r < ng.y; h1 = ng.x + r + R < ng.y;
                        if (h0) n0 = loadEdge<Codes>(m, ng.x + r, fc);
                        if (h1) n1 = loadEdge<Codes>(m, ng.x + r + R, fc);
                    }
                    if (k1) applyEdgePair<Dsm>(m, c0, c1, fc);
                    else if (k0) applyEdge<Dsm>(m, c0, fc);
                    for (int e = rg.x + r + 2 * R; e < rg.y; e += 2 * R) {
                        if (e + R < rg.y) applyEdgePair<Dsm>(m, loadEdge<Codes>(m, e, fc), loadEdge<Codes>(m, e + R, fc), fc);
                        else applyEdge<Dsm>(m, loadEdge<Codes>(m, e, fc), fc);
                    }
                } else {
                    for (int e = rg.x + r; e < rg.y; e += R) applyEdge<Dsm>(m, loadEdge<Codes>(m, e, fc), fc);
                }
                if (Ahead && c + 1 == m.nEdgeColors && fc.doStrain && !fc.doBend) loadFirstTet();
                if (!sync.sync()) return;
                mark(s, kPhaseEdges);
            }
        }
        if (fc.doBend)
            for (int c = 0; c < m.nBendColors; c++) {
                int2 rg = m.bendRange[c];
                for (int e = rg.x + r; e < rg.y; e += R) projectBend<Dsm>(m, e, fc);
                if (!sync.sync()) return;
                mark(s, kPhaseBends);
            }
        if (fc.doStrain) {
            if (!tetLoaded) loadFirstTet();
            for (int c = 0; c < m.nTetColors; c++) {
                int2 rg = m.tetRange[c];
                TetRecord cur = next;
                bool hasCur = hasNext;
                int2 nrg = c + 1 < m.nTetColors ? m.tetRange[c + 1] : make_int2(0, 0);
                hasNext = nrg.x + r < nrg.y;
                if (hasNext) next = loadTet<Codes>(m, nrg.x + r, fc);
                if (hasCur) applyTet<Dsm>(m, cur, fc, guarded);
                for (int k = rg.x + r + R; k < rg.y; k += R) projectTet<Dsm, Codes>(m, k, fc, guarded);
                if (!sync.sync()) return;
                mark(s, kPhaseTets);
            }
            if (guarded)   // tensile reinforcement after the tet colours (xpbd_solver.cu:2531-2533)
                for (int pass = 0; pass < fc.volumePasses; pass++)
                    for (int c = 0; c < m.nTetColors; c++) {
                        int2 rg = m.tetRange[c];
                        for (int k = rg.x + r; k < rg.y; k += R) projectTensile(m, k, fc, pass);
                        if (!sync.sync()) return;
                        mark(s, kPhaseTets);
                    }
        }
        // -- contact, velocity --
        float t = fminf(1.f, (float)(fc.firstSubstep + s + 1) / (float)fc.numSubsteps);
        ContactFrame cf;
        if (fc.contact && !m.nodeInstance) cf = contactFrame(from, to, t, cp, fc.contactAlphaH2);
        if (Extended && fc.friction) frictionPhase(m, fc, from, to, cp, t, r, R);   // contact model 1
        if (guarded) {   // contact, then the feasibility chain, then the velocity update
            if (fc.contact)
                for (int i = m.nodeBase + r; i < nodeEnd; i += R) contactNode(m, i, cf, cp);
            if (!guardFeasible(m, fc, fc.firstSubstep + s + 1, sync)) return;
        }
        // Without ⟂ damping or a blade the next substep's predict needs nothing but the node's own
        // state, so it follows each node's velocity update here, in registers (no barrier lies
        // between them anyway).  With Ahead a thread takes its nodes two at a time, loads ahead of
        // stores.
        predicted = s + 1 < fc.substeps && !fc.perpDamp && !fc.cut;
        const bool touch = fc.contact && !guarded;
        auto velocityNode = [&](int i, float4 P, float4 Q, float4 V, float4 F) {
            if (touch && P.w > 0.f) {
                const ContactFrame* own = &cf;   // batched instances: each node meets its own instance's tool
                if (m.nodeInstance) own = &m.contactFrames[(size_t)(fc.firstSubstep + s) * m.nInstances + m.nodeInstance[i]];
                const f3 p = contactPoint(xyz(P), P.w, xyz(V), *own, cp);
                P = make_float4(p.x, p.y, p.z, P.w);
            }
            f3 v = P.w > 0.f ? (xyz(P) - xyz(Q)) * fc.invH : mk(0.f, 0.f, 0.f);
            if (!fc.perpDamp) v = P.w > 0.f ? v * fc.velScale : mk(0.f, 0.f, 0.f);
            if (predicted && P.w > 0.f) {
                predictNode<Dsm>(m, i, P, v, F, fc.h);
                return;
            }
            m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
            if (predicted) predictNode<Dsm>(m, i, P, v, F, fc.h);
            else if (touch) posRef<Dsm>(m, i) = P;
        };
        // Colour 0 of the edges is a matching: a thread that runs this pass for both ends of a
        // colour-0 edge predicts the next substep for them and projects the edge on the spot, from
        // its registers, with the substep-start positions it just wrote as the damping term's.  Each
        // node and edge sees the operations it would see with a barrier between the two phases, in
        // the same order; the next substep starts its edge sweep at colour 1.
        const bool fuse = !Codes && !Dsm && !Extended && predicted && m.fuseEdge0 && fc.doEdges && m.nEdgeColors > 0;
        if (fuse) {
            auto velocityPredict = [&](int i, float4 P, float4 Q, float4 V, float4 F, f3& start) {
                if (touch && P.w > 0.f) {
                    const f3 p = contactPoint(xyz(P), P.w, xyz(V), cf, cp);
                    P = make_float4(p.x, p.y, p.z, P.w);
                }
                f3 v = P.w > 0.f ? (xyz(P) - xyz(Q)) * fc.invH : mk(0.f, 0.f, 0.f);
                v = P.w > 0.f ? v * fc.velScale : mk(0.f, 0.f, 0.f);
                if (!(P.w > 0.f)) m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
                start = xyz(P);
                return predictNode<Dsm>(m, i, P, v, F, fc.h);
            };
            FrameCoeffs noStart = fc;
            noStart.betaGammaHS = 0.f;   // the record's substep-start ends come from the registers below
            const int2 g0 = m.edgeRange[0];
            for (int e = g0.x + r; e < g0.y; e += R) {
                EdgeRecord er = loadEdge<false>(m, e, noStart);
                const int a = er.ij.x, b = er.ij.y;
                const float4 Pa = posRef<Dsm>(m, a), Qa = m.prev[a], Pb = posRef<Dsm>(m, b), Qb = m.prev[b];
                const float4 Va = touch ? m.vel[a] : make_float4(0.f, 0.f, 0.f, 0.f), Fa = m.ext[a];
                const float4 Vb = touch ? m.vel[b] : make_float4(0.f, 0.f, 0.f, 0.f), Fb = m.ext[b];
                const float4 Na = velocityPredict(a, Pa, Qa, Va, Fa, er.qi);
                const float4 Nb = velocityPredict(b, Pb, Qb, Vb, Fb, er.qj);
                float4 oa, ob;
                if (solveEdge(er, fc, Na, Nb, oa, ob)) {
                    posRef<Dsm>(m, a) = oa;
                    posRef<Dsm>(m, b) = ob;
                }
            }
            for (int q = r; q < m.nUncovered0; q += R) {
                const int i = m.uncovered0[q];
                const float4 Pi = posRef<Dsm>(m, i), Qi = m.prev[i];
                const float4 Vi = touch ? m.vel[i] : make_float4(0.f, 0.f, 0.f, 0.f), Fi = m.ext[i];
                f3 start;
                velocityPredict(i, Pi, Qi, Vi, Fi, start);
            }
            edge0Done = true;
        } else if (Codes && m.mobile) {
            for (int q = r; q < m.nMobile; q += R) {
                const int i = m.mobile[q];
                const float4 Pi = posRef<Dsm>(m, i), Qi = m.prev[i];
                const float4 Vi = touch ? m.vel[i] : make_float4(0.f, 0.f, 0.f, 0.f), Fi = predicted ? m.ext[i] : Vi;
                velocityNode(i, Pi, Qi, Vi, Fi);
            }
        } else
        for (int i = m.nodeBase + r; i < nodeEnd; i += (Ahead ? 2 : 1) * R) {
            const int j = Ahead ? i + R : nodeEnd;
            const float4 Pi = posRef<Dsm>(m, i), Qi = m.prev[i];
            const float4 Vi = touch ? m.vel[i] : make_float4(0.f, 0.f, 0.f, 0.f), Fi = predicted ? m.ext[i] : Vi;
            float4 Pj, Qj, Vj, Fj;
            if (j < nodeEnd) {
                Pj = posRef<Dsm>(m, j); Qj = m.prev[j];
                Vj = touch ? m.vel[j] : make_float4(0.f, 0.f, 0.f, 0.f); Fj = predicted ? m.ext[j] : Vj;
            }
            velocityNode(i, Pi, Qi, Vi, Fi);
            if (j < nodeEnd) velocityNode(j, Pj, Qj, Vj, Fj);
        }
        if (fc.perpDamp) {   // k_perp_damp_edges between the raw velocity write and the Rayleigh scale
            if (!sync.sync()) return;
            for (int c = 0; c < m.nEdgeColors; c++) {
                int2 rg = m.edgeRange[c];
                for (int e = rg.x + r; e < rg.y; e += R) {
                    int2 ij;
                    if (!edgeNodes<Codes>(m, e, ij)) continue;
                    float4 Pi = posRef<Dsm>(m, ij.x), Pj = posRef<Dsm>(m, ij.y);
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
            for (int i = m.nodeBase + r; i < nodeEnd; i += R) {
                float4 V = m.vel[i];
                f3 v = posRef<Dsm>(m, i).w > 0.f ? xyz(V) * fc.velScale : mk(0.f, 0.f, 0.f);
                m.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
            }
        }
        mark(s, kPhaseVelocity);
        // -- blade ribbon tick between substeps --
        if (fc.cut) {   // the first tick after the blade is set only takes the position snapshot
            if (havePrev) {
                // cut points emitted so far (the surface revision); nothing changes it between the
                // previous tick's closing barrier and this tick's opening one
                const unsigned pointsBefore = rotations ? *(volatile unsigned*)(cu.counters + 1) : 0u;
                if (!sync.sync()) return;
                const float* rot = rotations ? m.particleRot[rotParity] : nullptr;
                if (cu.brickList && cu.tearLen2 <= 0.f) {   // only the bricks near the blade
                    const int nb = ((m.dx + kBrick - 1) / kBrick) * ((m.dy + kBrick - 1) / kBrick) * ((m.dz + kBrick - 1) / kBrick);
                    for (int b = r >> 5; b < nb; b += R >> 5) brickBounds(m, cu, b, r & 31);
                    if (!sync.sync()) return;
                    mark(s, kPhaseTickBricks);
                    const int listed = min((int)*(volatile unsigned*)cu.brickCount, nb);
                    for (int j = r; j < listed * kBrickEdges; j += R) {
                        int4 g;
                        if (brickEdge(m, cu.brickList[j / kBrickEdges], j % kBrickEdges, g)) tickEdgeAt(m, cu, g, true, rot);
                    }
                } else {
                    for (int e = r; e < cu.nGridEdges; e += R) tickEdge(m, cu, e, true, rot);
                }
                if (!sync.sync()) return;
                if (sync.leader() && cu.brickCount) *cu.brickCount = 0u;   // every reader has passed the barrier above
                mark(s, kPhaseTick);
                // a tick that emitted cut points is followed by fresh frames before the next substep
                // (V/physics.cu:368-379)
                if (rotations && fc.firstSubstep + s + 1 < fc.numSubsteps && *(volatile unsigned*)(cu.counters + 1) != pointsBefore) {
                    framePass();
                    if (!sync.sync()) return;
                }
            }
            havePrev = true;
        }
    }
    if (rotations && fc.closingPass && fc.firstSubstep + fc.substeps == fc.numSubsteps) {   // LCS_Step's closing frames
        if (!sync.sync()) return;
        framePass();
    }
    if (sync.leader()) {
        *(volatile unsigned*)state = derivedAt;
        if (rotations) state[3] = (unsigned)rotParity;
    }
}

// Batched instances, one CTA per instance at a time: CTA b serves the instances
// order[ctaStart[b]] .. order[ctaStart[b+1]-1] (a longest-processing-time packing by tet count),
// each for the whole frame with __syncthreads between colours, on that instance's own colour
// ranges and node range of the packed table.  No grid barrier at all.
__device__ __forceinline__ void runInstances(const DeviceMesh& m, const FrameCoeffs& fc, const ContactParams& cp, const InstanceTable& it) {
    BlockSync b{nullptr};
    CutParams noCut{};
    ToolPose none{};
    for (int j = it.ctaStart[blockIdx.x]; j < it.ctaStart[blockIdx.x + 1]; j++) {
        const int i = it.order[j];
        DeviceMesh v = m;
        v.nodeBase = it.nodeBase[i];
        v.nNodes = it.nodeCount[i];
        v.edgeRange = it.edgeRange + (size_t)i * m.nEdgeColors;
        v.bendRange = it.bendRange + (size_t)i * m.nBendColors;
        v.tetRange = it.tetRange + (size_t)i * m.nTetColors;
        runFrame<BlockSync, false, false, false, 1, false, true>(v, fc, none, none, cp, noCut, it.derived + i, b);
        __syncthreads();
    }
}
// ---------------------------------------------------------------------------------------------
// batched instances on thread-block clusters: positions in distributed shared memory
// ---------------------------------------------------------------------------------------------
// Each cluster of K CTAs (512 threads each) runs its list of instances one after another.  An
// instance's positions are copied into the cluster's shared memory for the frame, interleaved in
// blocks of 512 nodes over the K CTAs (posRef<true>), which puts every node a thread updates in its
// own phases (predict, contact, velocity) in its own CTA; the colour sweeps gather and scatter the
// other nodes through distributed shared memory, and each colour ends at the hardware cluster
// barrier (release/acquire at cluster scope).  Everything else (prev, vel, element tables) stays in
// device memory.
struct ClusterSync {
    int r, n; bool lead;
    __device__ int rank() const { return r; }
    __device__ int spreadRank() const { return r; }
    __device__ int size() const { return n; }
    __device__ bool leader() const { return lead; }
    __device__ bool sync() { cooperative_groups::this_cluster().sync(); return true; }
};

__global__ void __launch_bounds__(kClusterThreads) frameKernelCluster(DeviceMesh m, FrameCoeffs fc, ContactParams cp, InstanceTable it,
                                                                       int logK) {
    extern __shared__ float4 clusterSlots[];
    __shared__ float4* bases[8];
    cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
    const int K = 1 << logK, rank = (int)cluster.block_rank();
    if ((int)threadIdx.x < K) bases[threadIdx.x] = cluster.map_shared_rank(clusterSlots, (int)threadIdx.x);
    __syncthreads();
    ClusterSync sync{rank * kClusterThreads + (int)threadIdx.x, K * kClusterThreads, rank == 0 && threadIdx.x == 0};
    const int cid = blockIdx.x >> logK;      // the CTAs of one cluster are consecutive in x
    CutParams noCut{};
    ToolPose none{};
    for (int j = it.ctaStart[cid]; j < it.ctaStart[cid + 1]; j++) {
        const int i = it.order[j];
        DeviceMesh v = m;
        v.nodeBase = it.nodeBase[i];
        v.nNodes = it.nodeCount[i];
        v.edgeRange = it.edgeRange + (size_t)i * m.nEdgeColors;
        v.bendRange = it.bendRange + (size_t)i * m.nBendColors;
        v.tetRange = it.tetRange + (size_t)i * m.nTetColors;
        v.dsm = bases; v.dsmLogB = kClusterLogThreads; v.dsmLogK = logK;
        for (int n = sync.r; n < v.nNodes; n += sync.n) posRef<true>(v, v.nodeBase + n) = m.pos[v.nodeBase + n];
        cluster.sync();
        runFrame<ClusterSync, false, true, false, 1, false, true>(v, fc, none, none, cp, noCut, it.derived + i, sync);
        cluster.sync();
        for (int n = sync.r; n < v.nNodes; n += sync.n) m.pos[v.nodeBase + n] = posRef<true>(v, v.nodeBase + n);
    }
    cluster.sync();   // no CTA leaves while another may still read its shared memory
}

// A single mesh on one thread-block cluster of 2^logK CTAs x kSessionClusterThreads: its positions in the
// cluster's distributed shared memory for the frame (as above), every phase closed by the hardware
// cluster barrier instead of a grid barrier.  Plain frames only (no blade tick, guard or friction;
// cu only supplies the topology revision);
// the closing particle-frame pass follows as its own launch, reading the parity word state[3].
__global__ void __launch_bounds__(kSessionClusterThreads, 1) frameKernelSessionCluster(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                              ContactParams cp, CutParams cu, unsigned* state, int logK) {
    extern __shared__ float4 clusterSlots[];
    __shared__ float4* bases[8];
    cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
    const int K = 1 << logK, rank = (int)cluster.block_rank();
    if ((int)threadIdx.x < K) bases[threadIdx.x] = cluster.map_shared_rank(clusterSlots, (int)threadIdx.x);
    __syncthreads();
    ClusterSync sync{rank * kSessionClusterThreads + (int)threadIdx.x, K * kSessionClusterThreads, rank == 0 && threadIdx.x == 0};
    DeviceMesh v = m;
    v.dsm = bases; v.dsmLogB = kSessionClusterLogThreads; v.dsmLogK = logK;
    for (int n = sync.r; n < v.nNodes; n += sync.n) posRef<true>(v, v.nodeBase + n) = m.pos[v.nodeBase + n];
    cluster.sync();
    runFrame<ClusterSync, false, true, true>(v, fc, from, to, cp, cu, state, sync);   // fc.cut is 0: no tick
    cluster.sync();
    for (int n = sync.r; n < v.nNodes; n += sync.n) m.pos[v.nodeBase + n] = posRef<true>(v, v.nodeBase + n);
    cluster.sync();   // no CTA leaves while another may still read its shared memory
}

__global__ void __launch_bounds__(256) frameKernelInstances256(DeviceMesh m, FrameCoeffs fc, ContactParams cp, InstanceTable it) {
    runInstances(m, fc, cp, it);
}
__global__ void __launch_bounds__(512) frameKernelInstances512(DeviceMesh m, FrameCoeffs fc, ContactParams cp, InstanceTable it) {
    runInstances(m, fc, cp, it);
}

template <bool Extended, int EdgeGroup, bool Ahead, bool Codes = false>
__device__ __forceinline__ void gridFrame(const DeviceMesh& m, const FrameCoeffs& fc, const ToolPose& from, const ToolPose& to,
                                          const ContactParams& cp, const CutParams& cu, unsigned* state) {
    GridSync g{state + 1, state + 2, gridDim.x, 0u, fc.spinBudget, (unsigned)fc.syncTestExtra};
    runFrame<GridSync, Extended, false, true, EdgeGroup, Ahead, Codes>(m, fc, from, to, cp, cu, state, g);
}
// A single mesh: one CTA per SM, so the tet projection keeps its registers without spilling (a
// colour of ~19 k tets still finds a warp for every scheduler).
__global__ void __launch_bounds__(kFrameThreads, 1) frameKernelGrid(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                  ContactParams cp, CutParams cu, unsigned* state) {
    gridFrame<false, 2, true>(m, fc, from, to, cp, cu, state);
}
// Batched instances in lockstep: two CTAs per SM (128 registers), since every colour of the packed
// table holds several elements per thread.
__global__ void __launch_bounds__(kFrameThreads, 2) frameKernelLockstep(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                     ContactParams cp, CutParams cu, unsigned* state) {
    gridFrame<false, 2, false, true>(m, fc, from, to, cp, cu, state);
}
__global__ void __launch_bounds__(kFrameThreads, 1) frameKernelGridExt(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                     ContactParams cp, CutParams cu, unsigned* state) {
    gridFrame<true, 2, false>(m, fc, from, to, cp, cu, state);
}

// One CTA per mesh.  When fc.stageNodes is set the whole node state (positions and substep-start
// positions, 32 B per node) is copied into shared memory for the frame, so every gather of every
// colour is a shared-memory access; it is written back when the frame ends.
template <bool Extended>
__device__ __forceinline__ void blockFrame(DeviceMesh m, const FrameCoeffs& fc, const ToolPose& from, const ToolPose& to,
                                           const ContactParams& cp, const CutParams& cu, unsigned* state) {
    extern __shared__ float4 staged[];
    BlockSync b{state + 2};
    if (!fc.stageNodes) {
        runFrame<BlockSync, Extended, false, true>(m, fc, from, to, cp, cu, state, b);
        return;
    }
    float4* sPos = staged;
    float4* sPrev = staged + m.nNodes;
    for (int i = threadIdx.x; i < m.nNodes; i += blockDim.x) { sPos[i] = m.pos[i]; sPrev[i] = m.prev[i]; }
    __syncthreads();
    float4* gPos = m.pos;
    float4* gPrev = m.prev;
    m.pos = sPos;
    m.prev = sPrev;
    runFrame<BlockSync, Extended, false, true>(m, fc, from, to, cp, cu, state, b);
    __syncthreads();
    for (int i = threadIdx.x; i < m.nNodes; i += blockDim.x) { gPos[i] = sPos[i]; gPrev[i] = sPrev[i]; }
}
__global__ void __launch_bounds__(kBlockThreads) frameKernelBlock(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                   ContactParams cp, CutParams cu, unsigned* state) {
    blockFrame<false>(m, fc, from, to, cp, cu, state);
}
__global__ void __launch_bounds__(kBlockThreads) frameKernelBlockExt(DeviceMesh m, FrameCoeffs fc, ToolPose from, ToolPose to,
                                                                      ContactParams cp, CutParams cu, unsigned* state) {
    blockFrame<true>(m, fc, from, to, cp, cu, state);
}

// One frame pass over every node, k_ComputeParticleRot (V/physics.cu:109-205): frames from
// particleRot[p] into particleRot[p ^ 1], p = *parityWord when given (the parity a frame kernel left
// on the device), else `parity`.
__global__ void particleRotKernel(DeviceMesh m, const unsigned* parityWord, int parity) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int p = parityWord ? (int)(*parityWord & 1u) : parity;
    if (c < m.nNodes) particleFrame(c, m.pos, m.nbr, m.active, m.pinned, m.particleRot[p], m.particleRot[p ^ 1]);
}

// Per-tet compliance of the frame, k_ComputeTetAlpha (xpbd_solver.cu:578-587).
__global__ void tetAlphaKernel(int n, float invH2, const float2* stiff, float2* alpha) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) { float2 s = stiff[k]; alpha[k] = make_float2(invH2 / s.x, invH2 / s.y); }
}

__global__ void packXyzKernel(int n, const float4* in, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = in[i];
    out[3 * i] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z;
}
__global__ void unpackXyzKernel(int n, const float* in, float4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = out[i];
    out[i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], v.w);
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

__global__ void detectQuadKernel(DeviceMesh m, CutParams cu, QuadTool tool, const float* rot) {
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
    markEdge(m, cu, rot, g, a, b, tr, O + D * tr, tool.ncut);
}

__global__ void __launch_bounds__(kFrameThreads) barrierFloorKernel(unsigned* sync, int barriers, long long budget) {
    GridSync g{sync, sync + 1, gridDim.x, 0u, budget, 0u};
    for (int k = 0; k < barriers; k++)
        if (!g.sync()) return;
}

__global__ void severKernel(DeviceMesh m, CutParams cu) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cu.nGridEdges) return;
    CutParams noTear = cu;
    noTear.tearLen2 = 0.f;
    tickEdge(m, noTear, e, false, nullptr);
}

}  // namespace gbt
