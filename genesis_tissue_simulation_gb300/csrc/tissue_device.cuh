// Device-side data layout and constraint projections of the XPBD tissue step.
//
// Layout in HBM (one mesh; the batched table holds one of these per instance):
//   node arrays, lattice order (id = x + nx*(y + ny*z)), one float4 per node:
//     pos  (x, y, z, inverse mass)   prev (x, y, z, 0)   vel (x, y, z, 0)   ext (body force xyz, mass)
//   tet table, colour order (the reference's greedy tet colouring, V/xpbd/xpbd_solver.cu:1738-1780):
//     tetIds int4, tetMeta int (Kuhn type | live << 3), tetAlpha float2
//     (deviatoric, hydrostatic compliance / h^2 of the frame), tetStiff float2 (mu*V, kappa*V)
//   edge table, colour order (greedy edge colouring, xpbd_solver.cu:1213-1249):
//     edgeEnds int2, edgeRest float, edgeOwner int (the 6p+s slot it was emitted from), edgeLive int
//   topology: nbr int[6N] (slot 2a = -a, 2a+1 = +a, -1 severed), bend pairs 32 B records.
//
// Every projection below evaluates the reference kernel's expression in the reference's operation
// order, with no contraction of multiply-add pairs (the library is compiled with -fmad=false), so
// results are rounded exactly as the CPU restatement rounds them.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbt {

struct BendRecord { int i, j, k; float theta0; int alive, p0, p1, p2; };
static_assert(sizeof(BendRecord) == 32, "BendPairGpu is 32 bytes");

struct ContactFrame;

// Everything a kernel needs about one mesh, or about the instances packed into one table.  Pointers
// are device memory.  The work of colour c is the element range [range[c].x, range[c].y) of the
// colour-ordered tables; nodes are [nodeBase, nodeBase + nNodes).  A single mesh has contiguous
// ranges; a batch stores all instances' colour-c members together (colour-major), and a kernel
// that serves one instance per CTA reads that instance's own ranges.
struct DeviceMesh {
    int nNodes, nodeBase, dx, dy, dz;       // nodes served, first node, voxel dims (single mesh)
    float4* pos; float4* prev; float4* vel; const float4* ext;
    const int* pinned; const int* active; int* nbr;
    // edges (colour order)
    int nEdgeColors; const int2* edgeRange;               // [nEdgeColors]
    const int2* edgeEnds; const float* edgeRest; const int* edgeOwner; int* edgeLive;
    // bends (colour order)
    int nBendColors; const int2* bendRange;
    const int4* bendIJK; const int* bendSrc; int* bendLive; BendRecord* bendPairs; int nBendPairs;
    // tets (colour order)
    int nTetColors; const int2* tetRange;                 // [nTetColors]
    const int4* tetIds; int* tetMeta; const int* tetOwner; float2* tetAlpha; const float2* tetStiff;
    int* edgeSupport;                                     // [6N] slot carried by a live tet
    // batched instances: the instance of every node and each instance's tool (previous, current)
    // (contactFrames: [substep][instance] instrument frames of the frame, evaluated on the host)
    const int* nodeInstance; const ContactFrame* contactFrames; int nInstances;
    float typeB[6][9];                                    // rest Dm^-1 of each Kuhn type, row major
};

// Per-frame coefficients, computed on the host in FP32 exactly as xpbd_begin_frame does
// (xpbd_solver.cu:2481-2514).
struct FrameCoeffs {
    int numSubsteps;                 // substeps of the frame (N, h = dt/N)
    int substeps, firstSubstep;      // substeps run by this launch, index of its first (0-based)
    int doEdges, fallback, doBend, doStrain, perpDamp, contact, cut;
    float h, invH, invH2, alphaTilde, betaGammaHS, alphaB, betaGammaHB, velScale, betaS;
    float omega, dampingOverH, fallbackInvEh2, contactAlphaH2;
    long long spinBudget;            // grid-barrier spin budget, SM clock cycles
    int syncTestExtra;               // > 0: barriers await arrivals that never come (timeout test)
    int stageNodes;                  // one-CTA kernel: node state staged in shared memory
    unsigned long long* phaseClock;  // optional: %globaltimer after every phase (section profiling)
};

// Phase tags of the section profiler; one 64-bit record per phase end: (tag << 56) | nanoseconds.
enum PhaseTag : unsigned { kPhaseFrameStart = 0, kPhasePredict = 1, kPhaseEdges = 2, kPhaseBends = 3, kPhaseTets = 4,
                           kPhaseVelocity = 5, kPhaseTick = 6 };
constexpr int kPhaseRecordsPerSubstep = 128;

// Shaft capsule + jaw slab of contact model 0 (XpbdToolState, xpbd_solver.h:223-229).
struct ToolPose { float sax, say, saz, sbx, sby, sbz, shaftR, hx, hy, hz, ax, ay, az, mx, my, mz, nx, ny, nz, halfWidth, len, gap, grasp01; };
static_assert(sizeof(ToolPose) == 92, "XpbdToolState is 92 bytes");
struct ContactParams { float jawGapClosed, contactAlpha, ccdVelThresh, ccdMaxDisp, ccdOmega; };

// Blade state of the ribbon tick (V/cut.cu:1303-1431).
struct CutParams {
    int nGridEdges; const int4* gridEdges; const unsigned* occupied; unsigned* cutMask;
    const int* inside; const float* skinT; float* edgeCutT; const float4* rest;
    unsigned* counters;   // [0] topology revision, [1] cut points, [2] tear marks
    float sx, sy, sz, ex, ey, ez;     // current blade segment S -> E
    float voxelL, tearLen2;
    int havePrev;
};

// ---------------------------------------------------------------------------------------------
// small float helpers (explicit operation order)
// ---------------------------------------------------------------------------------------------
// Host and device evaluate these identically: every operation is a single correctly rounded IEEE
// operation (the host side is compiled with -ffp-contract=off, the device side with -fmad=false).
#define GBT_HD __host__ __device__ __forceinline__
struct f3 { float x, y, z; };
GBT_HD f3 mk(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
GBT_HD f3 xyz(float4 a) { return mk(a.x, a.y, a.z); }
GBT_HD f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
GBT_HD f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
GBT_HD f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
GBT_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GBT_HD f3 cross(f3 a, f3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
GBT_HD float len(f3 a) { return sqrtf(dot(a, a)); }
GBT_HD float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Instrument frame of one substep, contact model 0 (xpbd_solver.cu:3467-3483, 3573-3580): the shaft
// capsule and jaw box interpolated linearly from the previous frame's command to the current one,
// the jaw frame orthonormalised.  `alpha` is the contact compliance over h^2.
struct ContactFrame { f3 sa, sb, hinge, axis, normal, w; float shaftR, jawLen, halfWidth, gapHalf, alpha; };
static_assert(sizeof(ContactFrame) == 92, "ContactFrame layout");
GBT_HD f3 lerpTool(float ax, float ay, float az, float bx, float by, float bz, float t) {
    return mk(ax, ay, az) * (1.f - t) + mk(bx, by, bz) * t;
}
GBT_HD ContactFrame contactFrame(const ToolPose& a, const ToolPose& b, float t, const ContactParams& cp, float alpha) {
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

// J^(-2/3): inverse cube root by four Newton steps in correction form y <- y + y(1 - J y^3)/3 from a
// bit-level seed (the exponent trick of the fast inverse square root applied to the -1/3 power,
// constant 0x54A23000 fitted on [0.05, 1e6]), squared.  <= 2.4 ulp from the exact power; the same
// sequence of correctly rounded operations runs on the host, so both sides agree bit for bit.
__device__ __forceinline__ float powMinusTwoThirds(float J) {
    unsigned bits = 0x54A23000u - __float_as_uint(J) / 3u;
    float y = __uint_as_float(bits);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float y3 = (y * y) * y;
        float r = 1.f - J * y3;
        y = y + (y * r) / 3.f;
    }
    return y * y;
}

// ---------------------------------------------------------------------------------------------
// constraint projections (one colour member each; members of a colour touch disjoint nodes)
// ---------------------------------------------------------------------------------------------
// What an edge projection reads that the sweep does not write (see TetRecord below).
struct EdgeRecord { int2 ij; int live; float rest; f3 qi, qj; };
__device__ __forceinline__ EdgeRecord loadEdge(const DeviceMesh& m, int e, const FrameCoeffs& fc) {
    EdgeRecord r;
    r.live = m.edgeLive[e];
    if (fc.fallback && r.live && m.edgeSupport[m.edgeOwner[e]]) r.live = 0;   // a live tet carries the edge
    r.ij = m.edgeEnds[e];
    r.rest = m.edgeRest[e];
    r.qi = xyz(m.prev[r.ij.x]);
    r.qj = xyz(m.prev[r.ij.y]);
    return r;
}

// Lattice-edge distance constraint, k_solve_edges (xpbd_solver.cu:484-524).  Multipliers restart
// at zero every substep and each edge is projected once, so the lambda term vanishes.
__device__ __forceinline__ void applyEdge(const DeviceMesh& m, const EdgeRecord& r, const FrameCoeffs& fc) {
    if (r.live == 0) return;
    float alphaTilde = fc.alphaTilde;
    if (fc.fallback) alphaTilde = fc.fallbackInvEh2 / r.rest;
    int2 ij = r.ij;
    float4 pi = m.pos[ij.x], pj = m.pos[ij.y];
    float wi = pi.w, wj = pj.w, ws = wi + wj;
    if (ws <= 0.f) return;
    f3 d = xyz(pi) - xyz(pj);
    float L = len(d);
    if (L < 1e-9f) return;
    f3 n = d * (1.f / L);
    float C = L - r.rest;
    float gamma = fc.betaGammaHS;
    float gradDx = dot(n, (xyz(pi) - r.qi) - (xyz(pj) - r.qj));
    float dl = (-C - gamma * gradDx) / ((1.f + gamma) * ws + alphaTilde);
    float ap = fc.omega * dl;
    f3 a = xyz(pi) + n * (wi * ap);
    f3 b = xyz(pj) - n * (wj * ap);
    m.pos[ij.x] = make_float4(a.x, a.y, a.z, wi);
    m.pos[ij.y] = make_float4(b.x, b.y, b.z, wj);
}

// Bending angle constraint, k_solve_bending (xpbd_solver.cu:534-573); off unless kb > 0.
__device__ __forceinline__ void projectBend(const DeviceMesh& m, int e, const FrameCoeffs& fc) {
    if (m.bendLive[e] == 0) return;
    int4 r = m.bendIJK[e];
    float4 Pi = m.pos[r.x], Pj = m.pos[r.y], Pk = m.pos[r.z];
    float wi = Pi.w, wj = Pj.w, wk = Pk.w;
    if (wi + wj + wk <= 0.f) return;
    f3 u = xyz(Pi) - xyz(Pj), v = xyz(Pi) - xyz(Pk);
    float Lu = len(u), Lv = len(v);
    if (Lu < 1e-9f || Lv < 1e-9f) return;
    f3 nu = u * (1.f / Lu), nv = v * (1.f / Lv);
    float c = fmaxf(-1.f, fminf(1.f, dot(nu, nv)));
    float s = sqrtf(fmaxf(1.f - c * c, 0.f));
    if (s < 1e-4f) return;
    float C = acosf(c) - __int_as_float(r.w);
    f3 gj = nv - nu * c, gk = nu - nv * c, gi = (gj + gk) * -1.f;
    float wg = wi * dot(gi, gi) + wj * dot(gj, gj) + wk * dot(gk, gk);
    float g = fc.betaGammaHB;
    f3 qi = xyz(m.prev[r.x]), qj = xyz(m.prev[r.y]), qk = xyz(m.prev[r.z]);
    float gdx = dot(gi, xyz(Pi) - qi) + dot(gj, xyz(Pj) - qj) + dot(gk, xyz(Pk) - qk);
    float den = (1.f + g) * wg + fc.alphaB;
    if (den < 1e-12f) return;
    float ap = fc.omega * ((-C - g * gdx) / den);
    f3 a = xyz(Pi) + gi * (wi * ap), b = xyz(Pj) + gj * (wj * ap), cc = xyz(Pk) + gk * (wk * ap);
    m.pos[r.x] = make_float4(a.x, a.y, a.z, wi);
    m.pos[r.y] = make_float4(b.x, b.y, b.z, wj);
    m.pos[r.z] = make_float4(cc.x, cc.y, cc.z, wk);
}

// What a tet projection reads that no phase of the Gauss-Seidel sweep writes: its record and the
// substep-start positions of its nodes.  Loading it ahead (before the barrier of the preceding
// colour) takes two dependent L2 round trips off each colour's critical path.
struct TetRecord { int4 ids; int meta; float2 alpha; f3 q[4]; };
__device__ __forceinline__ TetRecord loadTet(const DeviceMesh& m, int k) {
    TetRecord t;
    t.meta = m.tetMeta[k];
    t.ids = m.tetIds[k];
    t.alpha = m.tetAlpha[k];
    t.q[0] = xyz(m.prev[t.ids.x]); t.q[1] = xyz(m.prev[t.ids.y]); t.q[2] = xyz(m.prev[t.ids.z]); t.q[3] = xyz(m.prev[t.ids.w]);
    return t;
}

// Coupled deviatoric/hydrostatic Neo-Hookean block of one tet, k_solve_tet (xpbd_solver.cu:749-829),
// unguarded form (hydrostatic row J - 1, no trust region).
__device__ __forceinline__ void applyTet(const DeviceMesh& m, const TetRecord& t, const FrameCoeffs& fc) {
    int meta = t.meta;
    if ((meta & 8) == 0) return;
    const float* Bm = m.typeB[meta & 7];
    int id[4] = {t.ids.x, t.ids.y, t.ids.z, t.ids.w};
    float4 P[4] = {m.pos[id[0]], m.pos[id[1]], m.pos[id[2]], m.pos[id[3]]};
    f3 p[4] = {xyz(P[0]), xyz(P[1]), xyz(P[2]), xyz(P[3])};
    f3 br[3] = {mk(Bm[0], Bm[1], Bm[2]), mk(Bm[3], Bm[4], Bm[5]), mk(Bm[6], Bm[7], Bm[8])};
    f3 e1 = p[1] - p[0], e2 = p[2] - p[0], e3 = p[3] - p[0];
    f3 F[3];
#pragma unroll
    for (int c = 0; c < 3; c++) F[c] = e1 * comp(br[0], c) + e2 * comp(br[1], c) + e3 * comp(br[2], c);
    float I1 = dot(F[0], F[0]) + dot(F[1], F[1]) + dot(F[2], F[2]);
    f3 cof[3] = {cross(F[1], F[2]), cross(F[2], F[0]), cross(F[0], F[1])};
    float ad = t.alpha.x, ah = t.alpha.y;
    float J = dot(F[0], cof[0]), pJ = fmaxf(J, .05f);
    float iso = powMinusTwoThirds(pJ);
    float q = fmaxf(iso * I1 - 3.f, 0.f);
    float CD = sqrtf(fmaxf(q, 1e-12f));
    float devScale = 1.f / CD;
    float volGrad = J > .05f ? iso * I1 / (3.f * pJ) : 0.f;
    float CH = J - 1.f;
    f3 gd[4], gh[4];
#pragma unroll
    for (int c = 1; c < 4; c++) {
        f3 b = br[c - 1];
        gh[c] = cof[0] * b.x + cof[1] * b.y + cof[2] * b.z;
        gd[c] = ((F[0] * b.x + F[1] * b.y + F[2] * b.z) * iso - gh[c] * volGrad) * devScale;
    }
    gd[0] = (gd[1] + gd[2] + gd[3]) * -1.f;
    gh[0] = (gh[1] + gh[2] + gh[3]) * -1.f;
    float dd = 0.f, dh = 0.f, vd = 0.f, vh = 0.f, w[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        w[c] = P[c].w;
        dd += w[c] * dot(gd[c], gd[c]);
        dh += w[c] * dot(gd[c], gh[c]);
        f3 dx = p[c] - t.q[c];
        vd += dot(gd[c], dx);
        vh += dot(gh[c], dx);
    }
    float scale = 1.f + fc.dampingOverH, bulkScale = scale;
    float eAd = ad / scale, eAh = ah / bulkScale;
    float A = dd + eAd, Bc = dh, gamma = Bc / A;
    float schur = eAh + eAd * gamma * gamma;
#pragma unroll
    for (int c = 0; c < 4; c++) { f3 r = gh[c] - gd[c] * gamma; schur += w[c] * dot(r, r); }
    float rd = (-CD - fc.dampingOverH * vd) / scale;
    float rh = (-CH - (bulkScale - 1.f) * vh) / bulkScale;
    if (!(A > 0.f) || !(schur > 0.f)) return;
    float dlH = fc.omega * (rh - gamma * rd) / schur, dlD = (fc.omega * rd - Bc * dlH) / A;
    if (!isfinite(dlD) || !isfinite(dlH)) return;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        f3 o = p[c] + (gd[c] * dlD + gh[c] * dlH) * w[c];
        m.pos[id[c]] = make_float4(o.x, o.y, o.z, w[c]);
    }
}
__device__ __forceinline__ void projectTet(const DeviceMesh& m, int k, const FrameCoeffs& fc) { applyTet(m, loadTet(m, k), fc); }

// Liveness of one colour-ordered element from the live topology, k_RefreshLiveness
// (xpbd_solver.cu:429-466).
__device__ __forceinline__ void refreshEdge(const DeviceMesh& m, int e) {
    int2 ij = m.edgeEnds[e];
    m.edgeLive[e] = (m.nbr[m.edgeOwner[e]] >= 0 && m.active[ij.x] != 0 && m.active[ij.y] != 0) ? 1 : 0;
}
__device__ __forceinline__ void refreshTet(const DeviceMesh& m, int k) {
    const int* o = m.tetOwner + 3 * k;
    int4 d = m.tetIds[k];
    bool live = m.nbr[o[0]] >= 0 && m.nbr[o[1]] >= 0 && m.nbr[o[2]] >= 0 && m.active[d.x] != 0 && m.active[d.y] != 0 &&
                m.active[d.z] != 0 && m.active[d.w] != 0;
    int meta = m.tetMeta[k];
    m.tetMeta[k] = (meta & ~8) | (live ? 8 : 0);
}
__device__ __forceinline__ float nodeInvMass(const DeviceMesh& m, int i) {
    return (m.pinned[i] != 0 || m.active[i] == 0) ? 0.f : 1.f / m.ext[i].w;
}

}  // namespace gbt
