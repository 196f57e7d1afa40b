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
// order.  The compiler contracts nothing (the library is compiled with -fmad=false); the edge and tet
// projections contract chosen products into explicit fused multiply-adds (fmv, dotF, crossF, fmaf),
// and the CPU restatement calls std::fma at the same sites, so results round exactly as it rounds
// them.
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
    // tissue guard (armed by LCS_SetTissueGuard): per-tet fibre multipliers [6T], the feasibility
    // chain's candidate positions and marks [N], incident live-tet lists (CSR over colour slots),
    // and two flags (candidate below the minimum volume; still below after the repair)
    float* fiberLambda; float4* feasTarget; int* needed; const int* incOff; const int* incTet; unsigned* guardFlags;
    // instance positions in a cluster's distributed shared memory (cluster batch kernel): node j of
    // the instance (j = i - nodeBase) lives in CTA (j >> logB) & (K - 1), slot
    // ((j >> (logB + logK)) << logB) | (j & (B - 1)); dsm[k] is CTA k's array (a generic pointer)
    float4* const* dsm; int dsmLogB, dsmLogK;
    // particle frames (9 floats per node, rows of R): two buffers, current and previous, that
    // alternate on every frame pass
    float* particleRot[2];
    // debug builds (GBT_DEBUG_BOUNDS): out-of-range gather records [violations, first bad index,
    // site of the first]; null otherwise
    unsigned* bounds;
    // Batched lattices addressed implicitly (null: the explicit element tables above).  One 32-bit
    // code per element, colour order as the explicit tables -- a tet: local node of its corner 0
    // (bits 0-14), Kuhn type (15-17), live (18), instance (19-31); an edge: local node of its lower
    // end (0-14), axis (15-16), live (18), instance (19-31) -- and per instance its first node and
    // lattice strides (instGeo: base, nx, nx*ny, 0) and its six Kuhn types' compliances
    // (instAlpha[6 i + type]).  Every node of a tet or edge follows from the code, so a colour sweep
    // streams 4 B per element besides the edge rest lengths.
    unsigned* tetCode; unsigned* edgeCode; const int4* instGeo; const float2* instAlpha;
    // Batched lockstep grid: the nodes with a positive inverse mass, the only ones a node pass
    // changes (a node of inverse mass 0 keeps its position, substep-start position and zero velocity
    // from the start), so predict and velocity sweep this list; null: every node of the range.
    const int* mobile; int nMobile;
    // single sessions: the nodes that end no edge of colour 0 (colour 0 is a matching), for the
    // velocity pass that predicts the next substep and projects its colour-0 edges in one phase
    const int* uncovered0; int nUncovered0; int fuseEdge0;
};

// Corners a, b of Kuhn type t on its path 0 -> a -> b -> 7 (kKuhn in mesh_build.cu), 3 bits each,
// type t at bit 6t.
constexpr unsigned long long kKuhnPath = (1ull | 3ull << 3) | (3ull | 2ull << 3) << 6 | (2ull | 6ull << 3) << 12 |
                                         (6ull | 4ull << 3) << 18 | (4ull | 5ull << 3) << 24 | (5ull | 1ull << 3) << 30;
__host__ __device__ __forceinline__ int cornerOffset(unsigned corner, int nx, int nxy) {
    return (int)(corner & 1u) + ((corner >> 1) & 1u ? nx : 0) + ((corner >> 2) & 1u ? nxy : 0);
}
// The nodes of an implicit tet: corner 0 at n0, then its Kuhn path.
__host__ __device__ __forceinline__ int4 kuhnNodes(int type, int n0, int nx, int nxy) {
    const unsigned a = (unsigned)(kKuhnPath >> (6 * type)) & 7u, b = (unsigned)(kKuhnPath >> (6 * type + 3)) & 7u;
    return make_int4(n0, n0 + cornerOffset(a, nx, nxy), n0 + cornerOffset(b, nx, nxy), n0 + 1 + nx + nxy);
}
// The neighbour-table slots of an implicit tet's three lattice edges (a tet is live only while all
// three links are), in the order mesh_build.cu lists them.  The corners of type t form the lattice
// path 0 -> p -> q -> 7 with p one axis bit and q two; the Kuhn order visits q before p for types
// 1, 3 and 5.  Each edge is owned by its lower end's +axis slot (6 node + 2 axis + 1).
__host__ __device__ __forceinline__ void kuhnOwners(int type, int n0, int nx, int nxy, int o[3]) {
    const unsigned a = (unsigned)(kKuhnPath >> (6 * type)) & 7u, b = (unsigned)(kKuhnPath >> (6 * type + 3)) & 7u;
    const bool monotone = (a & (a - 1u)) == 0u;   // a is a single axis bit
    const unsigned p = monotone ? a : b, q = monotone ? b : a;
    auto axisOf = [](unsigned bit) { return bit == 1u ? 0 : bit == 2u ? 1 : 2; };
    o[0] = 6 * n0 + 2 * axisOf(p) + 1;
    o[1] = 6 * (n0 + cornerOffset(p, nx, nxy)) + 2 * axisOf(p ^ q) + 1;
    o[2] = 6 * (n0 + cornerOffset(q, nx, nxy)) + 2 * axisOf(q ^ 7u) + 1;
}
constexpr unsigned kCodeLive = 1u << 18;

// Gather-index checks of the debug build (GBT_DEBUG_BOUNDS, the stand-in for a memory checker):
// an element's node index outside the nodes the kernel serves, or a neighbour-table slot outside
// the table, is recorded in m.bounds and replaced by a valid index so the access stays in range.
// Release builds compile both to the index itself.
enum BoundsSite : unsigned { kSiteEdge = 1, kSiteBend = 2, kSiteTet = 3, kSiteEdgeSlot = 4, kSiteTetSlot = 5, kSiteNeighbour = 6 };
__device__ __forceinline__ void recordBounds(unsigned* rec, int index, unsigned site) {
    if (!rec) return;
    if (atomicAdd(rec, 1u) == 0u) { rec[1] = (unsigned)index; rec[2] = site; }
}
__device__ __forceinline__ int checkNode(const DeviceMesh& m, int i, unsigned site) {
#ifdef GBT_DEBUG_BOUNDS
    if ((unsigned)(i - m.nodeBase) >= (unsigned)m.nNodes) { recordBounds(m.bounds, i, site); return m.nodeBase; }
#else
    (void)m; (void)site;
#endif
    return i;
}
__device__ __forceinline__ int checkSlot(const DeviceMesh& m, int s, unsigned site) {
#ifdef GBT_DEBUG_BOUNDS
    if ((unsigned)(s - 6 * m.nodeBase) >= (unsigned)(6 * m.nNodes)) { recordBounds(m.bounds, s, site); return 6 * m.nodeBase; }
#else
    (void)m; (void)site;
#endif
    return s;
}

// A node's position: plain device memory, or its slot in the cluster's distributed shared memory.
template <bool Dsm>
__device__ __forceinline__ float4& posRef(const DeviceMesh& m, int i) {
    if (!Dsm) return m.pos[i];
    const int j = i - m.nodeBase;
    const int owner = (j >> m.dsmLogB) & ((1 << m.dsmLogK) - 1);
    const int slot = ((j >> (m.dsmLogB + m.dsmLogK)) << m.dsmLogB) | (j & ((1 << m.dsmLogB) - 1));
    return m.dsm[owner][slot];
}

// Per-frame coefficients, computed on the host in FP32 exactly as xpbd_begin_frame does
// (xpbd_solver.cu:2481-2514).
struct FrameCoeffs {
    int numSubsteps;                 // substeps of the frame (N, h = dt/N)
    int substeps, firstSubstep;      // substeps run by this launch, index of its first (0-based)
    int doEdges, fallback, doBend, doStrain, perpDamp, contact, cut;
    float h, invH, invH2, alphaTilde, betaGammaHS, alphaB, betaGammaHB, velScale, betaS;
    float omega, dampingOverH, fallbackInvEh2, contactAlphaH2;
    float invScale, invBulkScale;    // 1 / (1 + dampingOverH), 1 / (1 + bulkDampingOverH)
    int guarded, volumePasses;       // tissue guard: guarded tet form, tensile passes, feasibility chain
    float tensileStrength, bulkDampingOverH, minVolume;
    int friction;                    // contact model 1: tool SDFs, swept contact, Coulomb friction
    float muS, muD, jawThickness, contactRadius;
    int rotations, rotParity;        // particle frames after a tick that emitted cut points and, with
                                     // closingPass, after the frame; particleRot[rotParity] is current
    int closingPass;                 // 0: the host launches the closing frame pass on the whole GPU
    long long spinBudget;            // grid-barrier spin budget, SM clock cycles
    int syncTestExtra;               // > 0: barriers await arrivals that never come (timeout test)
    int stageNodes;                  // one-CTA kernel: node state staged in shared memory
    unsigned long long* phaseClock;  // optional: %globaltimer after every phase (section profiling)
};

// Phase tags of the section profiler; one 64-bit record per phase end: (tag << 56) | nanoseconds.
enum PhaseTag : unsigned { kPhaseFrameStart = 0, kPhasePredict = 1, kPhaseEdges = 2, kPhaseBends = 3, kPhaseTets = 4,
                           kPhaseVelocity = 5, kPhaseTick = 6, kPhaseTickBricks = 7 };
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
    // cut points (EmitCutPoint, V/cut.cu:186-215), one per directed lattice slot 6p + s of the owner
    // p: [2 (6p + s)] = offset from p on the undeformed edge plus the half-kerf, in p's frame (w = 1
    // once set); [2 (6p + s) + 1] = the outward cut normal in p's frame
    float4* cutRec;
    float toolD;          // blade thickness D
    float ncx, ncy, ncz;  // last valid world cut normal of the blade
    // brick pre-cull of the ribbon tick (null: every edge): listed bricks and their count, which
    // the tick leaves at zero
    int* brickList; unsigned* brickCount; int nBricks;
    int skipSevered;      // every live bend pair's two links exist (see the sever in the tick)
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
// Fused multiply-adds of the projections (one rounding each; the CPU restatement calls std::fma at
// the same sites, so both sides still round identically): a s + c, the dot product
// (a.x b.x + a.y b.y) + a.z b.z and the cross product, each with its products contracted.
GBT_HD f3 fmv(f3 a, float s, f3 c) { return mk(fmaf(a.x, s, c.x), fmaf(a.y, s, c.y), fmaf(a.z, s, c.z)); }
GBT_HD float dotF(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
GBT_HD f3 crossF(f3 a, f3 b) {
    return mk(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}

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

// J^(-2/3): inverse cube root by four Newton steps in correction form y <- y + y(1 - J y^3)(1/3) (both
// updates fused multiply-adds) from a
// bit-level seed (the exponent trick of the fast inverse square root applied to the -1/3 power,
// constant 0x54A23000 fitted on [0.05, 1e6]), squared.  <= 2.4 ulp from the exact power; the same
// sequence of correctly rounded operations runs on the host, so both sides agree bit for bit.
constexpr float kOneThird = 0.333333343f;   // 1/3 rounded to FP32
__device__ __forceinline__ float powMinusTwoThirds(float J) {
    unsigned bits = 0x54A23000u - __float_as_uint(J) / 3u;
    float y = __uint_as_float(bits);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float y3 = (y * y) * y;
        float r = fmaf(-J, y3, 1.f);
        y = fmaf(y * r, kOneThird, y);
    }
    return y * y;
}

// arccos c for the bending angle (c in [-1, 1]), by the half-angle reduction of the arcsine:
// |c| <= 1/2: acos c = pi/2 - asin c; c > 1/2: acos c = 2 asin s; c < -1/2: acos c = pi - 2 asin s,
// with s = sqrt((1 - |c|)/2) <= 1/2 (1 - |c| and the halving are exact there).  asin x = x + x z P(z),
// z = x^2 <= 1/4, P of degree 5 fitted by weighted least squares to (asin x - x)/(x z) on Chebyshev
// nodes of [0, 1/4] (oracle/fit_acos.py); pi/2 and pi as an FP32 head plus tail.  <= 1.1 ulp from the
// exact arccos; the CPU restatement evaluates the same sequence.
__device__ __forceinline__ float acosBend(float c) {
    const float a = fabsf(c);
    const bool mid = a <= 0.5f;
    const float z = mid ? c * c : (1.f - a) * 0.5f;
    const float x = mid ? c : sqrtf(z);
    float p = 0.03748363f;
    p = p * z + 0.014460857f;
    p = p * z + 0.03180234f;
    p = p * z + 0.044517495f;
    p = p * z + 0.075005025f;
    p = p * z + 0.1666666f;
    const float asinx = x + x * (z * p);
    if (mid) return 1.57079637f - (asinx - -4.37113883e-8f);
    return c > 0.f ? 2.f * asinx : 3.14159274f - (2.f * asinx - -8.74227766e-8f);
}

// log x for the guarded bulk strain (x >= 0.05, a positive normal float): x = m 2^e with m in
// (sqrt(1/2), sqrt(2)], log m = 2 atanh(s), s = (m - 1)/(m + 1), by its odd series to s^11 (the
// truncation is below 3e-9 relative), e ln 2 with ln 2 split into an exactly representable head
// and a tail.  The CPU restatement evaluates the same sequence.
__device__ __forceinline__ float logPositive(float x) {
    unsigned bits = __float_as_uint(x);
    int e = (int)(bits >> 23) - 127;
    float m = __uint_as_float((bits & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    float f = m - 1.f;                                  // exact on (sqrt(1/2), sqrt(2)]
    float s = f / (2.f + f), z = s * s;
    float t = z * (2.f / 11.f) + 2.f / 9.f;
    t = t * z + 2.f / 7.f;
    t = t * z + 2.f / 5.f;
    t = t * z + 2.f / 3.f;
    float r = s * (z * t) + s * 2.f;                    // 2s + s^3 (2/3 + 2 s^2 / 5 + ...)
    float fe = (float)e;
    return (r + fe * -2.12194440e-4f) + fe * 0.693359375f;
}

// ---------------------------------------------------------------------------------------------
// constraint projections (one colour member each; members of a colour touch disjoint nodes)
// ---------------------------------------------------------------------------------------------
// What an edge projection reads that the sweep does not write (see TetRecord below).
struct EdgeRecord { int2 ij; int live; float rest; f3 qi, qj; };
template <bool Codes = false>   // Codes: the kernel may meet implicit lattice codes (batched instances)
__device__ __forceinline__ EdgeRecord loadEdge(const DeviceMesh& m, int e, const FrameCoeffs& fc) {
    EdgeRecord r;
    if (Codes && m.edgeCode) {   // implicit lattice (no tet-support fallback there): ends from the code
        const unsigned code = m.edgeCode[e];
        const int4 g = m.instGeo[code >> 19];
        const int axis = (int)((code >> 15) & 3u), n0 = g.x + (int)(code & 0x7FFFu);
        r.live = (code & kCodeLive) ? 1 : 0;
        r.ij = make_int2(n0, n0 + (axis == 0 ? 1 : axis == 1 ? g.y : g.z));
    } else {
        r.live = m.edgeLive[e];
        if (fc.fallback && r.live && m.edgeSupport[checkSlot(m, m.edgeOwner[e], kSiteEdgeSlot)]) r.live = 0;   // a live tet carries the edge
        r.ij = m.edgeEnds[e];
    }
    r.ij.x = checkNode(m, r.ij.x, kSiteEdge); r.ij.y = checkNode(m, r.ij.y, kSiteEdge);
    r.rest = m.edgeRest[e];
    if (fc.betaGammaHS != 0.f) {   // substep-start ends: only the damping term reads them
        r.qi = xyz(m.prev[r.ij.x]);
        r.qj = xyz(m.prev[r.ij.y]);
    } else {
        r.qi = r.qj = mk(0.f, 0.f, 0.f);
    }
    return r;
}

// Lattice-edge distance constraint, k_solve_edges (xpbd_solver.cu:484-524).  Multipliers restart
// at zero every substep and each edge is projected once, so the lambda term vanishes.
// The projection of edge r from its end positions pi, pj: false when the edge is dead, has no
// mobile end or no length (nothing is written), else the new end positions.
__device__ __forceinline__ bool solveEdge(const EdgeRecord& r, const FrameCoeffs& fc, float4 pi, float4 pj, float4& oi, float4& oj) {
    if (r.live == 0) return false;
    float alphaTilde = fc.alphaTilde;
    if (fc.fallback) alphaTilde = fc.fallbackInvEh2 / r.rest;
    float wi = pi.w, wj = pj.w, ws = wi + wj;
    if (ws <= 0.f) return false;
    f3 d = xyz(pi) - xyz(pj);
    float L = sqrtf(dotF(d, d));
    if (L < 1e-9f) return false;
    f3 n = d * (1.f / L);
    float C = L - r.rest;
    float gamma = fc.betaGammaHS;
    // undamped (gamma = 0): the damping term is a zero and its gradient is not formed
    float num = gamma != 0.f ? fmaf(-gamma, dotF(n, (xyz(pi) - r.qi) - (xyz(pj) - r.qj)), -C) : -C;
    float dl = num / fmaf(1.f + gamma, ws, alphaTilde);
    float ap = fc.omega * dl;
    f3 a = fmv(n, wi * ap, xyz(pi));
    f3 b = fmv(n, -(wj * ap), xyz(pj));
    oi = make_float4(a.x, a.y, a.z, wi);
    oj = make_float4(b.x, b.y, b.z, wj);
    return true;
}
template <bool Dsm = false>
__device__ __forceinline__ void applyEdge(const DeviceMesh& m, const EdgeRecord& r, const FrameCoeffs& fc) {
    if (r.live == 0) return;
    float4 oi, oj;
    if (solveEdge(r, fc, posRef<Dsm>(m, r.ij.x), posRef<Dsm>(m, r.ij.y), oi, oj)) {
        posRef<Dsm>(m, r.ij.x) = oi;
        posRef<Dsm>(m, r.ij.y) = oj;
    }
}
// Two edges of one colour at once: members of a colour touch disjoint nodes, so both edges' ends
// are loaded before either is written and the two projections overlap.
template <bool Dsm = false>
__device__ __forceinline__ void applyEdgePair(const DeviceMesh& m, const EdgeRecord& r0, const EdgeRecord& r1, const FrameCoeffs& fc) {
    const float4 a0 = posRef<Dsm>(m, r0.ij.x), b0 = posRef<Dsm>(m, r0.ij.y);
    const float4 a1 = posRef<Dsm>(m, r1.ij.x), b1 = posRef<Dsm>(m, r1.ij.y);
    float4 oa0, ob0, oa1, ob1;
    const bool k0 = solveEdge(r0, fc, a0, b0, oa0, ob0), k1 = solveEdge(r1, fc, a1, b1, oa1, ob1);
    if (k0) { posRef<Dsm>(m, r0.ij.x) = oa0; posRef<Dsm>(m, r0.ij.y) = ob0; }
    if (k1) { posRef<Dsm>(m, r1.ij.x) = oa1; posRef<Dsm>(m, r1.ij.y) = ob1; }
}

// Bending angle constraint, k_solve_bending (xpbd_solver.cu:534-573); off unless kb > 0.
template <bool Dsm = false>
__device__ __forceinline__ void projectBend(const DeviceMesh& m, int e, const FrameCoeffs& fc) {
    if (m.bendLive[e] == 0) return;
    int4 r = m.bendIJK[e];
    r.x = checkNode(m, r.x, kSiteBend); r.y = checkNode(m, r.y, kSiteBend); r.z = checkNode(m, r.z, kSiteBend);
    float4 Pi = posRef<Dsm>(m, r.x), Pj = posRef<Dsm>(m, r.y), Pk = posRef<Dsm>(m, r.z);
    float wi = Pi.w, wj = Pj.w, wk = Pk.w;
    if (wi + wj + wk <= 0.f) return;
    f3 u = xyz(Pi) - xyz(Pj), v = xyz(Pi) - xyz(Pk);
    float Lu = len(u), Lv = len(v);
    if (Lu < 1e-9f || Lv < 1e-9f) return;
    f3 nu = u * (1.f / Lu), nv = v * (1.f / Lv);
    float c = fmaxf(-1.f, fminf(1.f, dot(nu, nv)));
    float s = sqrtf(fmaxf(1.f - c * c, 0.f));
    if (s < 1e-4f) return;
    float C = acosBend(c) - __int_as_float(r.w);
    f3 gj = nv - nu * c, gk = nu - nv * c, gi = (gj + gk) * -1.f;
    float wg = wi * dot(gi, gi) + wj * dot(gj, gj) + wk * dot(gk, gk);
    float g = fc.betaGammaHB;
    f3 qi = xyz(m.prev[r.x]), qj = xyz(m.prev[r.y]), qk = xyz(m.prev[r.z]);
    float gdx = dot(gi, xyz(Pi) - qi) + dot(gj, xyz(Pj) - qj) + dot(gk, xyz(Pk) - qk);
    float den = (1.f + g) * wg + fc.alphaB;
    if (den < 1e-12f) return;
    float ap = fc.omega * ((-C - g * gdx) / den);
    f3 a = xyz(Pi) + gi * (wi * ap), b = xyz(Pj) + gj * (wj * ap), cc = xyz(Pk) + gk * (wk * ap);
    posRef<Dsm>(m, r.x) = make_float4(a.x, a.y, a.z, wi);
    posRef<Dsm>(m, r.y) = make_float4(b.x, b.y, b.z, wj);
    posRef<Dsm>(m, r.z) = make_float4(cc.x, cc.y, cc.z, wk);
}

// What a tet projection reads that no phase of the Gauss-Seidel sweep writes: its record and the
// substep-start positions of its nodes.  Loading it ahead (before the barrier of the preceding
// colour) takes two dependent L2 round trips off each colour's critical path.
struct TetRecord { int4 ids; int meta; float2 alpha; f3 q[4]; };
// Whether the tet projection has a damping term (Kelvin-Voigt strain damping, or the guarded
// form's bulk damping); without one the substep-start positions are neither loaded nor used.
__device__ __forceinline__ bool tetDamped(const FrameCoeffs& fc, bool guarded) {
    return fc.dampingOverH != 0.f || (guarded && fc.bulkDampingOverH != 0.f);
}
template <bool Codes = false>
__device__ __forceinline__ TetRecord loadTet(const DeviceMesh& m, int k, const FrameCoeffs& fc) {
    TetRecord t;
    if (Codes && m.tetCode) {   // implicit lattice: nodes from the code, compliances per instance and Kuhn type
        const unsigned code = m.tetCode[k];
        const int inst = (int)(code >> 19), type = (int)((code >> 15) & 7u);
        const int4 g = m.instGeo[inst];
        t.ids = kuhnNodes(type, g.x + (int)(code & 0x7FFFu), g.y, g.z);
        t.meta = type | ((code & kCodeLive) ? 8 : 0);
        t.alpha = m.instAlpha[6 * inst + type];
    } else {
        t.meta = m.tetMeta[k];
        t.ids = m.tetIds[k];
        t.alpha = m.tetAlpha[k];
    }
    t.ids.x = checkNode(m, t.ids.x, kSiteTet); t.ids.y = checkNode(m, t.ids.y, kSiteTet);
    t.ids.z = checkNode(m, t.ids.z, kSiteTet); t.ids.w = checkNode(m, t.ids.w, kSiteTet);
    if (tetDamped(fc, fc.guarded != 0)) {
        t.q[0] = xyz(m.prev[t.ids.x]); t.q[1] = xyz(m.prev[t.ids.y]); t.q[2] = xyz(m.prev[t.ids.z]); t.q[3] = xyz(m.prev[t.ids.w]);
    } else {
        t.q[0] = t.q[1] = t.q[2] = t.q[3] = mk(0.f, 0.f, 0.f);
    }
    return t;
}

// Coupled deviatoric/hydrostatic Neo-Hookean block of one tet, k_solve_tet (xpbd_solver.cu:749-829).
// Unguarded: hydrostatic row J - 1.  Guarded (tissue guard armed): row log J with a linear floor
// below J = 0.05, its own bulk damping, and a trust region capping every corner's move at 0.15 over
// the longest row of Dm^-1.
template <bool Dsm = false>
__device__ __forceinline__ void applyTet(const DeviceMesh& m, const TetRecord& t, const FrameCoeffs& fc, bool guardedForm = false) {
    int meta = t.meta;
    if ((meta & 8) == 0) return;
    const float* Bm = m.typeB[meta & 7];
    int id[4] = {t.ids.x, t.ids.y, t.ids.z, t.ids.w};
    float4 P[4] = {posRef<Dsm>(m, id[0]), posRef<Dsm>(m, id[1]), posRef<Dsm>(m, id[2]), posRef<Dsm>(m, id[3])};
    f3 p[4] = {xyz(P[0]), xyz(P[1]), xyz(P[2]), xyz(P[3])};
    f3 br[3] = {mk(Bm[0], Bm[1], Bm[2]), mk(Bm[3], Bm[4], Bm[5]), mk(Bm[6], Bm[7], Bm[8])};
    f3 e1 = p[1] - p[0], e2 = p[2] - p[0], e3 = p[3] - p[0];
    f3 F[3];
#pragma unroll
    for (int c = 0; c < 3; c++) F[c] = fmv(e3, comp(br[2], c), fmv(e2, comp(br[1], c), e1 * comp(br[0], c)));
    float I1 = dotF(F[0], F[0]) + dotF(F[1], F[1]) + dotF(F[2], F[2]);
    f3 cof[3] = {crossF(F[1], F[2]), crossF(F[2], F[0]), crossF(F[0], F[1])};
    float ad = t.alpha.x, ah = t.alpha.y;
    float J = dotF(F[0], cof[0]), pJ = fmaxf(J, .05f);
    float iso = powMinusTwoThirds(pJ);
    float q = fmaxf(fmaf(iso, I1, -3.f), 0.f);
    float CD = sqrtf(fmaxf(q, 1e-12f));
    float devScale = 1.f / CD;
    float volGrad = J > .05f ? iso * I1 / (3.f * pJ) : 0.f;
    const bool guarded = guardedForm;   // a compile-time false in the kernels built without the tissue guard
    float CH = guarded ? logPositive(pJ) + fminf(0.f, (J - .05f) / .05f) : J - 1.f;
    f3 gd[4], gh[4];
#pragma unroll
    for (int c = 1; c < 4; c++) {
        f3 b = br[c - 1];
        gh[c] = fmv(cof[2], b.z, fmv(cof[1], b.y, cof[0] * b.x));
        gd[c] = fmv(fmv(F[2], b.z, fmv(F[1], b.y, F[0] * b.x)), iso, gh[c] * -volGrad) * devScale;
        if (guarded) gh[c] = gh[c] * (1.f / pJ);
    }
    gd[0] = (gd[1] + gd[2] + gd[3]) * -1.f;
    gh[0] = (gh[1] + gh[2] + gh[3]) * -1.f;
    // undamped: the velocity terms vd, vh enter multiplied by zero and are not formed
    const bool damped = tetDamped(fc, guarded);
    float dd = 0.f, dh = 0.f, vd = 0.f, vh = 0.f, w[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        w[c] = P[c].w;
        dd = fmaf(w[c], dotF(gd[c], gd[c]), dd);
        dh = fmaf(w[c], dotF(gd[c], gh[c]), dh);
        if (damped) {
            f3 dx = p[c] - t.q[c];
            vd += dotF(gd[c], dx);
            vh += dotF(gh[c], dx);
        }
    }
    // 1 / (1 + D/h) is a frame constant; one reciprocal of A serves gamma and dlD
    float bulkScale = guarded ? 1.f + fc.bulkDampingOverH : 1.f + fc.dampingOverH;
    float invScale = fc.invScale, invBulk = guarded ? fc.invBulkScale : fc.invScale;
    float eAd = ad * invScale, eAh = ah * invBulk;
    float A = dd + eAd, invA = 1.f / A, Bc = dh, gamma = Bc * invA;
    float schur = fmaf(eAd * gamma, gamma, eAh);
#pragma unroll
    for (int c = 0; c < 4; c++) { f3 r = fmv(gd[c], -gamma, gh[c]); schur = fmaf(w[c], dotF(r, r), schur); }
    float rd = damped ? fmaf(-fc.dampingOverH, vd, -CD) * invScale : -CD * invScale;
    float rh = damped ? fmaf(-(bulkScale - 1.f), vh, -CH) * invBulk : -CH * invBulk;
    if (!(A > 0.f) || !(schur > 0.f)) return;
    float dlH = fc.omega * fmaf(-gamma, rd, rh) / schur, dlD = fmaf(-Bc, dlH, fc.omega * rd) * invA;
    if (!isfinite(dlD) || !isfinite(dlH)) return;
    if (guarded) {
        float largest = 0.f;
#pragma unroll
        for (int c = 0; c < 4; c++) largest = fmaxf(largest, len(fmv(gd[c], dlD, gh[c] * dlH) * w[c]));
        float limit = .15f / fmaxf(len(br[0]), fmaxf(len(br[1]), len(br[2])));
        float accepted = largest > limit ? limit / largest : 1.f;
        dlD *= accepted; dlH *= accepted;
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        f3 o = fmv(fmv(gd[c], dlD, gh[c] * dlH), w[c], p[c]);
        posRef<Dsm>(m, id[c]) = make_float4(o.x, o.y, o.z, w[c]);
    }
}
template <bool Dsm = false, bool Codes = false>
__device__ __forceinline__ void projectTet(const DeviceMesh& m, int k, const FrameCoeffs& fc, bool guardedForm = false) {
    applyTet<Dsm>(m, loadTet<Codes>(m, k, fc), fc, guardedForm);
}

// Liveness of one colour-ordered element from the live topology, k_RefreshLiveness
// (xpbd_solver.cu:429-466).
// The two nodes of edge e and whether it is live (either table form).
template <bool Codes = false>
__device__ __forceinline__ bool edgeNodes(const DeviceMesh& m, int e, int2& ij) {
    if (Codes && m.edgeCode) {
        const unsigned code = m.edgeCode[e];
        const int4 g = m.instGeo[code >> 19];
        const int axis = (int)((code >> 15) & 3u), n0 = g.x + (int)(code & 0x7FFFu);
        ij = make_int2(checkNode(m, n0, kSiteEdge), checkNode(m, n0 + (axis == 0 ? 1 : axis == 1 ? g.y : g.z), kSiteEdge));
        return (code & kCodeLive) != 0;
    }
    ij = make_int2(checkNode(m, m.edgeEnds[e].x, kSiteEdge), checkNode(m, m.edgeEnds[e].y, kSiteEdge));
    return m.edgeLive[e] != 0;
}
template <bool Codes = false>
__device__ __forceinline__ void refreshEdge(const DeviceMesh& m, int e) {
    if (Codes && m.edgeCode) {   // the link's own slot, 6 (lower end) + 2 axis + 1
        const unsigned code = m.edgeCode[e];
        const int4 g = m.instGeo[code >> 19];
        const int axis = (int)((code >> 15) & 3u);
        const int i = checkNode(m, g.x + (int)(code & 0x7FFFu), kSiteEdge);
        const int j = checkNode(m, i + (axis == 0 ? 1 : axis == 1 ? g.y : g.z), kSiteEdge);
        const bool live = m.nbr[checkSlot(m, 6 * i + 2 * axis + 1, kSiteEdgeSlot)] >= 0 && m.active[i] != 0 && m.active[j] != 0;
        m.edgeCode[e] = live ? (code | kCodeLive) : (code & ~kCodeLive);
        return;
    }
    int2 ij = m.edgeEnds[e];
    ij.x = checkNode(m, ij.x, kSiteEdge); ij.y = checkNode(m, ij.y, kSiteEdge);
    m.edgeLive[e] = (m.nbr[checkSlot(m, m.edgeOwner[e], kSiteEdgeSlot)] >= 0 && m.active[ij.x] != 0 && m.active[ij.y] != 0) ? 1 : 0;
}
template <bool Codes = false>
__device__ __forceinline__ void refreshTet(const DeviceMesh& m, int k) {
    int4 d; int o0, o1, o2;
    unsigned code = 0;
    if (Codes && m.tetCode) {   // the three lattice edges of the tet's Kuhn path
        code = m.tetCode[k];
        const int type = (int)((code >> 15) & 7u);
        const int4 g = m.instGeo[code >> 19];
        const int n0 = g.x + (int)(code & 0x7FFFu);
        d = kuhnNodes(type, n0, g.y, g.z);
        int o[3];
        kuhnOwners(type, n0, g.y, g.z, o);
        o0 = o[0]; o1 = o[1]; o2 = o[2];
    } else {
        const int* o = m.tetOwner + 3 * k;
        d = m.tetIds[k];
        o0 = o[0]; o1 = o[1]; o2 = o[2];
    }
    d.x = checkNode(m, d.x, kSiteTet); d.y = checkNode(m, d.y, kSiteTet); d.z = checkNode(m, d.z, kSiteTet); d.w = checkNode(m, d.w, kSiteTet);
    o0 = checkSlot(m, o0, kSiteTetSlot); o1 = checkSlot(m, o1, kSiteTetSlot); o2 = checkSlot(m, o2, kSiteTetSlot);
    bool live = m.nbr[o0] >= 0 && m.nbr[o1] >= 0 && m.nbr[o2] >= 0 && m.active[d.x] != 0 && m.active[d.y] != 0 &&
                m.active[d.z] != 0 && m.active[d.w] != 0;
    if (Codes && m.tetCode) {
        m.tetCode[k] = live ? (code | kCodeLive) : (code & ~kCodeLive);
        return;
    }
    int meta = m.tetMeta[k];
    m.tetMeta[k] = (meta & ~8) | (live ? 8 : 0);
}
__device__ __forceinline__ float nodeInvMass(const DeviceMesh& m, int i) {
    return (m.pinned[i] != 0 || m.active[i] == 0) ? 0.f : 1.f / m.ext[i].w;
}

// ---------------------------------------------------------------------------------------------
// tissue guard (xpbd_solver.cu:588-741), armed by LCS_SetTissueGuard with passes > 0
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void typeRows(const DeviceMesh& m, int type, f3 b[3]) {
    const float* B = m.typeB[type];
    b[0] = mk(B[0], B[1], B[2]); b[1] = mk(B[3], B[4], B[5]); b[2] = mk(B[6], B[7], B[8]);
}

// Tensile reinforcement of one live tet (projectTensile, xpbd_solver.cu:592-620): each of the six
// corner-to-corner fibres carries mu V strength / 2 s^6, s = max(length / rest - 1, 0), projected
// with finite compliance alphaDev / strength; the rest corners are the columns of (Dm^-1)^-1.
// `pass` > 0 continues the fibres' multipliers of this substep.
__device__ __forceinline__ void projectTensile(const DeviceMesh& m, int k, const FrameCoeffs& fc, int pass) {
    int meta = m.tetMeta[k];
    if ((meta & 8) == 0 || !(fc.tensileStrength > 0.f)) return;
    int4 ids = m.tetIds[k];
    int id[4] = {ids.x, ids.y, ids.z, ids.w};
    float4 P[4] = {m.pos[id[0]], m.pos[id[1]], m.pos[id[2]], m.pos[id[3]]};
    f3 p[4] = {xyz(P[0]), xyz(P[1]), xyz(P[2]), xyz(P[3])};
    f3 b[3];
    typeRows(m, meta & 7, b);
    float detB = dot(b[0], cross(b[1], b[2]));
    f3 rest[4] = {mk(0.f, 0.f, 0.f), cross(b[1], b[2]) * (1.f / detB), cross(b[2], b[0]) * (1.f / detB), cross(b[0], b[1]) * (1.f / detB)};
    float alpha = m.tetAlpha[k].x / fmaxf(fc.tensileStrength, 1e-10f);
    int fiber = 0;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = i + 1; j < 4; j++, fiber++) {
            f3 edge = p[j] - p[i];
            float length = len(edge), restLength = len(rest[j] - rest[i]);
            float strain = fmaxf(length / restLength - 1.f, 0.f), gradient = 3.f * strain * strain / restLength;
            float wi = P[i].w, wj = P[j].w;
            float lambda = pass == 0 ? 0.f : m.fiberLambda[6 * (size_t)k + fiber];
            if (strain > 0.f && length > 0.f) {
                float dl = (-strain * strain * strain - alpha * lambda) / ((wi + wj) * gradient * gradient + alpha);
                f3 g = edge * (gradient / length);
                lambda += dl;
                p[i] = p[i] - g * (wi * dl);
                p[j] = p[j] + g * (wj * dl);
            }
            if (fc.volumePasses > 1) m.fiberLambda[6 * (size_t)k + fiber] = lambda;
        }
#pragma unroll
    for (int c = 0; c < 4; c++) m.pos[id[c]] = make_float4(p[c].x, p[c].y, p[c].z, P[c].w);
}

// Relative volume det(Ds) det(Dm^-1) of colour slot k at the current positions.
__device__ __forceinline__ float tetVolume(const DeviceMesh& m, int k, int meta) {
    int4 ids = m.tetIds[k];
    f3 b[3];
    typeRows(m, meta & 7, b);
    f3 a = xyz(m.pos[ids.x]), u = xyz(m.pos[ids.y]) - a, v = xyz(m.pos[ids.z]) - a, w = xyz(m.pos[ids.w]) - a;
    return dot(u, cross(v, w)) * dot(b[0], cross(b[1], b[2]));
}

// Linearised volume repair of one live tet below minimum + 1e-4 (k_RepairMinimumVolume).
__device__ __forceinline__ void repairTet(const DeviceMesh& m, int k, float minimum) {
    int meta = m.tetMeta[k];
    if ((meta & 8) == 0) return;
    int4 ids = m.tetIds[k];
    int id[4] = {ids.x, ids.y, ids.z, ids.w};
    float4 P[4] = {m.pos[id[0]], m.pos[id[1]], m.pos[id[2]], m.pos[id[3]]};
    f3 p[4] = {xyz(P[0]), xyz(P[1]), xyz(P[2]), xyz(P[3])};
    f3 b[3];
    typeRows(m, meta & 7, b);
    f3 u = p[1] - p[0], v = p[2] - p[0], w = p[3] - p[0];
    float detB = dot(b[0], cross(b[1], b[2]));
    float J = dot(u, cross(v, w)) * detB;
    if (!isfinite(J) || J >= minimum + 1e-4f) return;
    f3 g[4];
    g[1] = cross(v, w) * detB; g[2] = cross(w, u) * detB; g[3] = cross(u, v) * detB;
    g[0] = (g[1] + g[2] + g[3]) * -1.f;
    float den = 0.f;
#pragma unroll
    for (int c = 0; c < 4; c++) den += P[c].w * dot(g[c], g[c]);
    if (den < 1e-20f) return;
    float dl = (minimum + 2e-4f - J) / den;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        f3 o = p[c] + g[c] * (P[c].w * dl);
        m.pos[id[c]] = make_float4(o.x, o.y, o.z, P[c].w);
    }
}

// Whether a live tet's motion over the substep (substep-start positions `prev` to the candidate)
// may pass below minimum + 1e-5 (k_NeedFeasible): a conservative bound first, then the 16 corners
// of the multi-affine volume; if so its four corners are marked.
__device__ __forceinline__ void needFeasible(const DeviceMesh& m, int k, float minimum) {
    int meta = m.tetMeta[k];
    if ((meta & 8) == 0) return;
    int4 ids = m.tetIds[k];
    int id[4] = {ids.x, ids.y, ids.z, ids.w};
    f3 x[4], d[4];
#pragma unroll
    for (int c = 0; c < 4; c++) { x[c] = xyz(m.prev[id[c]]); d[c] = xyz(m.pos[id[c]]) - x[c]; }
    f3 b[3];
    typeRows(m, meta & 7, b);
    float detB = dot(b[0], cross(b[1], b[2]));
    f3 u = x[1] - x[0], vv = x[2] - x[0], w = x[3] - x[0];
    float r0 = len(d[0]), r1 = r0 + len(d[1]), r2 = r0 + len(d[2]), r3 = r0 + len(d[3]);
    float bound = r1 * len(cross(vv, w)) + r2 * len(cross(w, u)) + r3 * len(cross(u, vv)) + r1 * r2 * len(w) + r1 * r3 * len(vv) +
                  r2 * r3 * len(u) + r1 * r2 * r3;
    if (dot(u, cross(vv, w)) * detB - bound * fabsf(detB) >= minimum + 1e-5f) return;
    bool bad = false;
    for (int mask = 0; mask < 16 && !bad; mask++) {
        f3 p[4];
#pragma unroll
        for (int c = 0; c < 4; c++) p[c] = x[c] + d[c] * (float)((mask >> c) & 1);
        float j = dot(p[1] - p[0], cross(p[2] - p[0], p[3] - p[0])) * detB;
        if (!isfinite(j) || j < minimum + 1e-5f) bad = true;
    }
    if (bad)
#pragma unroll
        for (int c = 0; c < 4; c++) m.needed[id[c]] = 1;
}

// One marked vertex advances from its substep-start position towards its candidate as far as every
// incident live tet keeps its volume above min(minimum, current) (k_FeasibleVertex); the volume is
// linear in this vertex's displacement with the other three fixed.
__device__ __forceinline__ void feasibleVertex(const DeviceMesh& m, int i, float minimum) {
    if (!m.needed[i]) return;
    float4 Pi = m.pos[i];
    f3 delta = xyz(m.feasTarget[i]) - xyz(Pi);
    float accepted = 1.f;
    if (!isfinite(delta.x + delta.y + delta.z)) return;
    for (int q = m.incOff[i]; q < m.incOff[i + 1]; q++) {
        int k = m.incTet[q];
        int meta = m.tetMeta[k];
        if ((meta & 8) == 0) continue;
        int4 ids = m.tetIds[k];
        f3 b[3];
        typeRows(m, meta & 7, b);
        f3 a = xyz(m.pos[ids.x]), u = xyz(m.pos[ids.y]) - a, v = xyz(m.pos[ids.z]) - a, w = xyz(m.pos[ids.w]) - a;
        float detB = dot(b[0], cross(b[1], b[2]));
        float j = dot(u, cross(v, w)) * detB;
        f3 grad[3] = {cross(v, w), cross(w, u), cross(u, v)};
        f3 g = i == ids.x ? (grad[0] + grad[1] + grad[2]) * -1.f : i == ids.y ? grad[0] : i == ids.z ? grad[1] : grad[2];
        float dj = dot(g, delta) * detB;
        if (dj < 0.f) {
            float floorV = fminf(minimum, fmaxf(0.f, j));
            if (j + dj < floorV) accepted = fminf(accepted, fmaxf(0.f, .95f * (j - floorV) / (-dj)));
        }
    }
    f3 o = xyz(Pi) + delta * accepted;
    m.pos[i] = make_float4(o.x, o.y, o.z, Pi.w);
}

}  // namespace gbt
