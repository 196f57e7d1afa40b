// CPU ORACLE — test infrastructure only.  Nothing in the product links or calls this file; the
// tests and __graft_entry__.smoke() load it to check the CUDA library against it, and bench.py's
// CPU-baseline leg times it.
//
// A plain restatement, on the CPU, of the reference's plain XPBD tissue step and its geometric
// cut, exporting the same LCS_* C ABI as the reference plugin
// (endoscopic_tissue/native/vendor/src/plugin_api.cpp) so one Python harness drives the oracle,
// the CUDA library and (on a machine with a GPU) the reference build identically.
//
// Built three times from this one source:
//   liboracle_f32.so  ORACLE_REAL=float   FP32, the arithmetic the reference performs, in the CUDA
//                     library's operation order (frame-constant reciprocals, one reciprocal of the 2x2
//                     pivot, an own J^(-2/3) and log), so the library matches it bit for bit
//   liboracle_f32w.so ORACLE_REAL=float, ORACLE_AS_WRITTEN: the tet projection exactly as the
//                     reference writes it (its divisions, the library power and logarithm), the
//                     independent anchor for every arithmetic rewrite of the CUDA path
//   liboracle_f64.so  ORACLE_REAL=double  FP64 accuracy oracle (same algorithm, double throughout)
// Both compile with -ffp-contract=off so results are identical on x86-64 and aarch64 hosts.
// OpenMP parallelises each colour (members of one colour touch disjoint nodes, so the order
// inside a colour does not change results); it is also the timed CPU baseline.
//
// Reference files followed ("V/" = endoscopic_tissue/native/vendor/cuda/):
//   V/physics.cu:214-315 (physics_init), 317-329 (gravity), 331-394 (physics_step),
//     109-205 + 399-411 particle frames (frames_oracle.inc)
//   V/dc_recon.cu:97-455, 469-487, 507-541 dual-contouring surface (surface_oracle.inc)
//   V/xpbd/xpbd_solver.cu:393-412 predict, 429-466 liveness, 469-479 tet edge support,
//     484-524 edges, 534-573 bending, 578-587 tet alpha, 749-829 tets, 871-919 velocity,
//     1049-1123 CCD capsule/jaw contact, 1204-1279 edge colouring, 1332-1400 bend colouring,
//     1412-1577 bind, 1600-1848 tet build, 2327-2472 set_tool, 2481-2514 begin_frame,
//     3460-3721 substep (plain branch)
//   V/cut.cu:186-254 MarkAndEmit, 421-474 DetectCutQuad, 486-592 DetectCutCCD,
//     607-681 TearOverstretch, 719-746 SeverLinks, 1105-1226 init/set_tool,
//     1235-1254 detect, 1303-1431 ribbon tick;  V/cut.cuh:113-188 lattice helpers, Moller-Trumbore
//   V/dc_recon.cu:543-620 (recon_init: positions, rest snapshot, skin crossing fractions)
//   cut_topology_oracle.inc: the library's cut-topology product (no reference counterpart)
#include <algorithm>
#include <array>
#include <chrono>
#include <map>
#include <climits>
#include <cstdint>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL Real;

#define API extern "C" __attribute__((visibility("default")))

// ---------------------------------------------------------------------------------------------
// ABI structs (byte layouts of the reference; sizes asserted)
// ---------------------------------------------------------------------------------------------
struct F3 { float x, y, z; };
struct ReconInitDesc { int voxelCount, cornerCount, isectCount, surfaceEdgeCount, triCapacity, dimsX, dimsY, dimsZ; float L; int qefIters; };
struct PhysicsInitDesc { int cornerCount, bendPairCount; float ks, cs, kb, cb, hInit, hMax; int maxSubsteps; float alpha, youngE, poisson, strainDamping; };
struct CutInitDesc { int voxelCount, cornerCount, gridEdgeCount, isectCount, triCapacity, dimsX, dimsY, dimsZ; float voxelL, originX, originY, originZ; int cutPointCapacity; float cutFPInterp, tearStretchRatio; };
struct CutToolDesc { float t1v0[3], t1v1[3], t1v2[3], t2v0[3], t2v1[3], t2v2[3], ncut[3]; float d; int valid; float aabbMin[3], aabbMax[3]; };
struct XpbdToolState { F3 shaftA, shaftB; float shaftR; F3 jawHinge, jawAxis, jawMid, jawNormal; float jawHalfWidth, jawLen, jawGap, grasp01; };
struct XpbdGraspParams { float graspThreshold, releaseThreshold, jawGapClosed, coreEllipseFrac, mu, contactAlpha, contactSkin, ccdVelThresh, ccdMaxDisp, ccdOmega, omegaGrasp, coreAlpha, coreBreakForce, graspMaxDisp; int nExemptRings; };
struct BendPair { int i, j, k; float theta0; int alive, p0, p1, p2; };
struct GridEdge2 { int axis, bx, by, bz; };
struct IsectRec { F3 pos, nrm; int a, b; float t; int insideA; };
static_assert(sizeof(ReconInitDesc) == 40, "ReconInitDesc");
static_assert(sizeof(PhysicsInitDesc) == 52, "PhysicsInitDesc");
static_assert(sizeof(CutInitDesc) == 60, "CutInitDesc");
static_assert(sizeof(CutToolDesc) == 116, "CutToolDesc");
static_assert(sizeof(XpbdToolState) == 92, "XpbdToolState");
static_assert(sizeof(XpbdGraspParams) == 60, "XpbdGraspParams");
static_assert(sizeof(BendPair) == 32, "BendPair");
static_assert(sizeof(IsectRec) == 40, "IsectRec");

enum {
    ERR_NOT_READY = -1000, ERR_NO_FRAME = -1001, ERR_BAD_DT = -1002, ERR_COLOR_OVERFLOW = -1003,
    ERR_BAD_ARG = -1004, ERR_IRREGULAR_REST = -1005, ERR_UNSUPPORTED = -4001,
};

// ---------------------------------------------------------------------------------------------
// vector helpers in Real
// ---------------------------------------------------------------------------------------------
struct V3 { Real x, y, z; };
static inline V3 v3(Real x, Real y, Real z) { V3 r = {x, y, z}; return r; }
static inline V3 fromF(const F3& a) { return v3(a.x, a.y, a.z); }
static inline V3 fromA(const float* a) { return v3(a[0], a[1], a[2]); }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, Real s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline Real dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline Real len(V3 a) { return std::sqrt(dot(a, a)); }
// The fused multiply-adds the CUDA library's edge and tet projections use (std::fma: one rounding,
// as the device's fmaf), at the same sites; the as-written build evaluates the same expressions
// unfused, which is exactly the reference's order (a s + c and c + a s round alike).
#ifdef ORACLE_AS_WRITTEN
static inline Real fmaR(Real a, Real b, Real c) { return a * b + c; }
#else
static inline Real fmaR(Real a, Real b, Real c) { return std::fma(a, b, c); }
#endif
static inline V3 fmv(V3 a, Real s, V3 c) { return v3(fmaR(a.x, s, c.x), fmaR(a.y, s, c.y), fmaR(a.z, s, c.z)); }
static inline Real dotF(V3 a, V3 b) { return fmaR(a.z, b.z, fmaR(a.y, b.y, a.x * b.x)); }
static inline V3 crossF(V3 a, V3 b) {
    return v3(fmaR(a.y, b.z, -(a.z * b.y)), fmaR(a.z, b.x, -(a.x * b.z)), fmaR(a.x, b.y, -(a.y * b.x)));
}
static inline Real comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static inline bool isFin(Real x) { return std::isfinite(x); }

// J^(-2/3) for the deviatoric invariant.  FP32: inverse cube root by Newton's method in correction
// form, y <- y + y(1 - J y^3)/3, four steps from a bit-level seed (the exponent trick of the fast
// inverse square root applied to the -1/3 power, seed constant 0x54A23000 fitted on [0.05, 1e6]),
// then squared: <= 2.4 ulp from the exact power.  The CUDA kernels evaluate the same operation
// sequence, so both sides round identically.  FP64: the library power function.
static inline float powMinusTwoThirds(float J) {
    uint32_t bits;
    std::memcpy(&bits, &J, 4);
    bits = 0x54A23000u - bits / 3u;
    float y;
    std::memcpy(&y, &bits, 4);
    for (int k = 0; k < 4; k++) {
        float y3 = (y * y) * y;
        float r = std::fma(-J, y3, 1.f);
        y = std::fma(y * r, 0.333333343f, y);   // 1/3 rounded to FP32
    }
    return y * y;
}
static inline double powMinusTwoThirds(double J) { return std::pow(J, -2.0 / 3.0); }

// arccos c for the bending angle (c in [-1, 1]).  FP32: the half-angle reduction of the arcsine
// (|c| <= 1/2: pi/2 - asin c; c > 1/2: 2 asin s; c < -1/2: pi - 2 asin s; s = sqrt((1 - |c|)/2)),
// asin x = x + x z P(z), z = x^2, P of degree 5 fitted by least squares (fit_acos.py), pi/2 and pi
// as head plus tail; <= 1.1 ulp; the CUDA kernels evaluate the same sequence.  FP64: the library
// arccos.
static inline float acosBend(float c) {
    const float a = std::fabs(c);
    const bool mid = a <= 0.5f;
    const float z = mid ? c * c : (1.f - a) * 0.5f;
    const float x = mid ? c : std::sqrt(z);
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
static inline double acosBend(double c) { return std::acos(c); }

// log x for the guarded bulk strain (x >= 0.05, a positive normal float).  FP32: x = m 2^e with
// m in (sqrt(1/2), sqrt(2)], log m = 2 atanh(s), s = (m - 1)/(m + 1), by its odd series to s^11,
// e ln 2 with ln 2 split into an exact head and a tail; the CUDA kernels evaluate the same sequence.
// FP64: the library logarithm.
static inline float logPositive(float x) {
    uint32_t bits;
    std::memcpy(&bits, &x, 4);
    int e = (int)(bits >> 23) - 127;
    bits = (bits & 0x007FFFFFu) | 0x3F800000u;
    float m;
    std::memcpy(&m, &bits, 4);
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
static inline double logPositive(double x) { return std::log(x); }

// ---------------------------------------------------------------------------------------------
// session state (one process-global session, as in the reference plugin)
// ---------------------------------------------------------------------------------------------
struct Session {
    // reconstruction-owned shared corner grid
    bool reconReady = false;
    int N = 0, dx = 0, dy = 0, dz = 0;
    std::vector<V3> pos, rest;
    std::vector<float> skinT;                 // [6N] skin crossing fraction per directed edge slot
    // physics
    bool physReady = false;
    PhysicsInitDesc pd = {};
    std::vector<Real> mass;
    std::vector<int> pinned, active, nbr;     // nbr [6N]
    std::vector<V3> ext, vel, prev;           // ext = body force (gravity * mass)
    std::vector<BendPair> bends;
    // xpbd params
    int numSubsteps = 20; Real ks = 0, kb = 0, alpha = 0, betaS = 0, betaB = 0, youngE = 0, poisson = 0.45, strainDamping = 0;
    Real omega = 1, damping = 0;
    // colour-ordered edges
    int E = 0; std::vector<int> eI, eJ, eOwner, eActive; std::vector<Real> eRest; std::vector<int> eColOff, eColCnt;
    // colour-ordered bends
    int B = 0; std::vector<int> bI, bJ, bK, bSrc, bActive; std::vector<Real> bTheta; std::vector<int> bColOff, bColCnt;
    // tets in storage order (Kuhn type major, cell minor)
    int T = 0; std::vector<int> tIds, tOwner, tActive, tColorOrder, tColOff, tColCnt, tType;
    Real typeB[6][3][3]; std::vector<Real> muV, kappaV, aDev, aHyd;
    std::vector<int> edgeSupport;             // [6N]
    std::vector<Real> invMass;
    std::vector<Real> particleRot, particleRotPrev;   // [9N] particle frames, rows of R
    std::vector<Real> cutRec;                         // [8 x 6N] cut point per directed slot: local xyz w, normal xyz
    std::vector<int> conn;                            // [9 x 4096] connectivity table (Conn4096Gpu)
    bool livenessStale = true; unsigned livenessRevision = 0xffffffffu;
    // frame
    bool frameReady = false; Real h = 0, alphaTilde = 0, velScale = 1, betaGammaHS = 0, alphaB = 0, betaGammaHB = 0;
    bool doBend = false, doStrain = false; int substepIndex = 0;
    float bulkDampingSeconds = 0.003125f, tissueHardening = 80.f; int volumePasses = 0;
    // tissue guard (LCS_SetTissueGuard): minimum relative volume, per-node incident tets, feasibility state
    Real minVolume = 0; std::vector<int> incOff, incTet, needed; std::vector<V3> feasTarget; std::vector<Real> fiberLambda;
    long long guardStats[3] = {0, 0, 0};   // substeps with a candidate below the minimum; still below after repair; marked vertices
    // tool / contact (contact model 0: capsule + jaw slab CCD gate)
    bool toolArmed = false, grasping = false; XpbdToolState tool = {}, toolFrom = {};
    XpbdGraspParams gp = {0.5f, 0.3f, 0.02f, 0.55f, 0.3f, 1.0e-7f, 0.02f, 0.5f, 0.045f, 0.25f, 0.25f, 1.0e-7f, 150.f, 0.045f, 1};
    int contactModel = 0;
    Real muStatic = 0, muDynamic = 0, jawThickness = 0, contactRadius = 0;   // contact model 1 (LCS_SetContactModel)
    std::vector<Real> jawLambda, shaftLambda;
    // cut
    bool cutReady = false; CutInitDesc cd = {}; std::vector<GridEdge2> gridEdges; std::vector<unsigned> occupied, cutMask;
    std::vector<int> inside; std::vector<V3> prevCorner; std::vector<float> edgeCutT;
    unsigned cutPoints = 0, revision = 0, tearMarks = 0;
    bool toolSet = false, havePrev = false, pressure = false; CutToolDesc cutTool = {}; V3 emitNcut = {0, 1, 0};
    Real tearLen2 = 0; std::vector<int> edgeWasExempt, edgeDecay;
    // profiling
    bool profile = false; std::vector<double> stepMs;
};
static Session S;

static int cid(int x, int y, int z) { return x + (S.dx + 1) * (y + (S.dy + 1) * z); }
#include "frames_oracle.inc"

// ---------------------------------------------------------------------------------------------
// greedy colouring: first free colour (< 64) not used by any member vertex (xpbd_solver.cu:1213-1230)
// ---------------------------------------------------------------------------------------------
template <int K>
static int greedyColour(int count, const int* members, int nodes, std::vector<int>& colour, int& numColours) {
    std::vector<uint64_t> used(nodes, 0);
    colour.assign(count, 0); numColours = 0;
    for (int e = 0; e < count; e++) {
        uint64_t u = 0;
        for (int k = 0; k < K; k++) u |= used[members[K * e + k]];
        int c = 0;
        while (c < 64 && (u >> c & 1)) c++;
        if (c >= 64) return ERR_COLOR_OVERFLOW;
        colour[e] = c;
        for (int k = 0; k < K; k++) used[members[K * e + k]] |= 1ull << c;
        numColours = std::max(numColours, c + 1);
    }
    return 0;
}
// bucket elements by colour: offsets/counts and the element at each colour-ordered slot
static void bucket(const std::vector<int>& colour, int numColours, std::vector<int>& off, std::vector<int>& cnt, std::vector<int>& slotOf) {
    cnt.assign(numColours, 0);
    for (int c : colour) cnt[c]++;
    off.assign(numColours, 0);
    for (int c = 1; c < numColours; c++) off[c] = off[c - 1] + cnt[c - 1];
    std::vector<int> cur = off;
    slotOf.assign(colour.size(), 0);
    for (size_t e = 0; e < colour.size(); e++) slotOf[e] = cur[colour[e]]++;
}

static void resetPhysics() {
    // a live physics session's shutdown restores the tissue material defaults (physics.cu:218 ->
    // xpbd_shutdown, xpbd_solver.cu:3829); a material set before the first LCS_InitPhysics stays
    if (S.physReady) { S.tissueHardening = 80.f; S.bulkDampingSeconds = 0.003125f; }
    S.physReady = false; S.frameReady = false; S.E = S.B = S.T = 0; S.toolArmed = false; S.grasping = false;
    S.livenessStale = true; S.livenessRevision = 0xffffffffu;
    S.volumePasses = 0; S.minVolume = 0; S.incOff.clear(); S.incTet.clear(); S.h = 0;
}
static void resetCut() { S.cutReady = false; S.toolSet = false; S.havePrev = false; S.cutPoints = S.revision = S.tearMarks = 0; }

// ---------------------------------------------------------------------------------------------
// LCS_Init — recon_init subset: the shared corner grid, its rest snapshot and skin crossings
// ---------------------------------------------------------------------------------------------
static int slotOfDirected(int a, int b) {
    int d = b - a, ad = d < 0 ? -d : d;
    int axis = ad == 1 ? 0 : (ad == S.dx + 1 ? 1 : 2);
    return 6 * a + 2 * axis + (d > 0 ? 1 : 0);
}
#include "surface_oracle.inc"
API int LCS_Init(const ReconInitDesc* desc, const float* cornerPos, const int* voxelCorner, const int* voxelIsectOffset,
                 const int* voxelIsectCount, const void* isect, const void* surfaceEdges) {
    resetCut(); resetPhysics(); S.reconReady = false; SS = SurfaceState();
    if (!desc) return -1000;
    int vc = desc->voxelCount, cc = desc->cornerCount;
    if (vc <= 0 || cc <= 0 || desc->triCapacity <= 0 || !cornerPos) return -1001;
    if ((long long)(desc->dimsX + 1) * (desc->dimsY + 1) * (desc->dimsZ + 1) != cc) return -1001;
    S.N = cc; S.dx = desc->dimsX; S.dy = desc->dimsY; S.dz = desc->dimsZ;
    S.pos.resize(cc); S.rest.resize(cc);
    for (int i = 0; i < cc; i++) S.pos[i] = S.rest[i] = v3(cornerPos[3 * i], cornerPos[3 * i + 1], cornerPos[3 * i + 2]);
    S.skinT.assign((size_t)6 * cc, -1.f);
    const IsectRec* is = (const IsectRec*)isect;
    for (int i = 0; is && i < desc->isectCount; i++) {
        S.skinT[slotOfDirected(is[i].a, is[i].b)] = is[i].t;
        S.skinT[slotOfDirected(is[i].b, is[i].a)] = 1.f - is[i].t;
    }
    S.reconReady = true;
    if (voxelCorner) {   // the static surface of the rest lattice and its rest snapshot
        int rc = initSurfaceO(desc, voxelCorner, voxelIsectOffset, voxelIsectCount, is, (const int*)surfaceEdges);
        if (rc) { S.reconReady = false; SS = SurfaceState(); return rc; }
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------
// LCS_InitPhysics — physics_init + xpbd_bind + xpbd_build_tets
// ---------------------------------------------------------------------------------------------
static bool inv3(const double m[3][3], double o[3][3]) {
    double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                 m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    if (std::fabs(det) < 1e-20) return false;
    double id = 1.0 / det;
    o[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id; o[0][1] = -(m[0][1] * m[2][2] - m[0][2] * m[2][1]) * id;
    o[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id; o[1][0] = -(m[1][0] * m[2][2] - m[1][2] * m[2][0]) * id;
    o[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id; o[1][2] = -(m[0][0] * m[1][2] - m[0][2] * m[1][0]) * id;
    o[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id; o[2][1] = -(m[0][0] * m[2][1] - m[0][1] * m[2][0]) * id;
    o[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    return true;
}
static double det3(const double m[3][3]) {
    return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}
static const int KUHN[6][4] = {{0, 1, 3, 7}, {0, 3, 2, 7}, {0, 2, 6, 7}, {0, 6, 4, 7}, {0, 4, 5, 7}, {0, 5, 1, 7}};

static int buildTets() {
    const int cc = S.N;
    double sp[3] = {((double)(float)S.pos[cid(S.dx, 0, 0)].x - (double)(float)S.pos[0].x) / S.dx,
                    ((double)(float)S.pos[cid(0, S.dy, 0)].y - (double)(float)S.pos[0].y) / S.dy,
                    ((double)(float)S.pos[cid(0, 0, S.dz)].z - (double)(float)S.pos[0].z) / S.dz};
    double tB[6][3][3], tV[6];
    for (int ti = 0; ti < 6; ti++) {
        double Dm[3][3];
        for (int k = 1; k < 4; k++)
            for (int a = 0; a < 3; a++) Dm[a][k - 1] = ((KUHN[ti][k] >> a) & 1) * sp[a];
        if (!inv3(Dm, tB[ti])) return ERR_IRREGULAR_REST;
        tV[ti] = std::fabs(det3(Dm)) / 6.0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) S.typeB[ti][a][b] = (Real)tB[ti][a][b];
    }
    // material: mu = E/(2(1+nu)), kappa = E/(3(1-2nu)) in float as the reference (xpbd_solver.cu:1636-1644)
    float E = (float)S.youngE, nu = (float)S.poisson, muF, kF;
    if (E > 0.f && nu > -1.f && nu < 0.5f) { muF = E / (2.f * (1.f + nu)); kF = E / (3.f * (1.f - 2.f * nu)); }
    else { muF = kF = 1.f; }
    if (!(muF > 0.f)) muF = 1.f;
    if (!(kF > 0.f)) kF = 1.f;

    std::vector<int> ids, owner, type; std::vector<Real> mv, kv;
    for (int z = 0; z < S.dz; z++)
        for (int y = 0; y < S.dy; y++)
            for (int x = 0; x < S.dx; x++) {
                bool all = true;
                for (int li = 0; li < 8 && all; li++)
                    if (!S.active[cid(x + (li & 1), y + (li >> 1 & 1), z + (li >> 2 & 1))]) all = false;
                if (!all) continue;
                for (int ti = 0; ti < 6; ti++) {
                    int g[4]; V3 p[4];
                    for (int k = 0; k < 4; k++) {
                        int l = KUHN[ti][k];
                        g[k] = cid(x + (l & 1), y + (l >> 1 & 1), z + (l >> 2 & 1));
                        p[k] = S.rest[g[k]];
                    }
                    double Dm[3][3], Bm[3][3];
                    for (int c = 0; c < 3; c++) {
                        V3 e = p[c + 1] - p[0];
                        double ed[3] = {(double)(float)p[c + 1].x - (double)(float)p[0].x, (double)(float)p[c + 1].y - (double)(float)p[0].y,
                                        (double)(float)p[c + 1].z - (double)(float)p[0].z};
                        (void)e;
                        for (int a = 0; a < 3; a++) Dm[a][c] = ed[a];
                    }
                    if (!inv3(Dm, Bm)) continue;
                    if (std::fabs(det3(Dm)) / 6.0 < 1e-12) continue;
                    double scale = 0, dev = 0;
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) {
                            scale = std::max(scale, std::fabs(tB[ti][a][b]));
                            dev = std::max(dev, std::fabs(Bm[a][b] - tB[ti][a][b]));
                        }
                    if (dev > 1e-4 * scale) return ERR_IRREGULAR_REST;
                    int found = 0;
                    for (int a = 0; a < 4 && found < 3; a++)
                        for (int b = a + 1; b < 4 && found < 3; b++) {
                            int lu = KUHN[ti][a], lv = KUHN[ti][b], d = lu ^ lv;
                            if (d != 1 && d != 2 && d != 4) continue;
                            int axis = d == 1 ? 0 : (d == 2 ? 1 : 2);
                            int lower = ((lu >> axis) & 1) == 0 ? lu : lv;
                            owner.push_back(6 * cid(x + (lower & 1), y + (lower >> 1 & 1), z + (lower >> 2 & 1)) + 2 * axis + 1);
                            found++;
                        }
                    for (int k = 0; k < 4; k++) ids.push_back(g[k]);
                    if (sizeof(Real) == 4) { mv.push_back((Real)(muF * (float)tV[ti])); kv.push_back((Real)(kF * (float)tV[ti])); }
                    else { mv.push_back((Real)((double)muF * tV[ti])); kv.push_back((Real)((double)kF * tV[ti])); }
                    type.push_back(ti);
                }
            }
    const int T = (int)type.size();
    std::vector<int> colour; int nc = 0;
    int rc = greedyColour<4>(T, ids.data(), cc, colour, nc);
    if (rc) return rc;
    // storage place: Kuhn type major, emission (cell) order minor (xpbd_solver.cu:1762-1780)
    std::vector<int> place(T), cursor(7, 0);
    for (int e = 0; e < T; e++) cursor[type[e] + 1]++;
    for (int k = 1; k < 7; k++) cursor[k] += cursor[k - 1];
    for (int e = 0; e < T; e++) place[e] = cursor[type[e]]++;
    std::vector<int> slotOf;
    bucket(colour, nc, S.tColOff, S.tColCnt, slotOf);
    S.T = T;
    S.tIds.assign((size_t)4 * T, 0); S.tOwner.assign((size_t)3 * T, 0); S.tType.assign(T, 0);
    S.muV.assign(T, 0); S.kappaV.assign(T, 0); S.tColorOrder.assign(T, 0);
    for (int e = 0; e < T; e++) {
        int d = place[e];
        for (int k = 0; k < 4; k++) S.tIds[4 * d + k] = ids[4 * e + k];
        for (int k = 0; k < 3; k++) S.tOwner[3 * d + k] = owner[3 * e + k];
        S.tType[d] = type[e]; S.muV[d] = mv[e]; S.kappaV[d] = kv[e];
        S.tColorOrder[slotOf[e]] = d;
    }
    if (T % 6) return ERR_IRREGULAR_REST;
    S.tActive.assign(T, 1); S.aDev.assign(T, 0); S.aHyd.assign(T, 0);
    S.edgeSupport.assign((size_t)6 * cc, 0);
    return 0;
}

API int LCS_InitPhysics(const PhysicsInitDesc* desc, const float* mass, const int* pinned, const int* active, const float* extForce,
                        const int* nbrIdx, const float* restNbr, const void* bendPairs) {
    resetPhysics();
    if (!desc) return -2000;
    if (!std::isfinite(desc->youngE) || desc->youngE < 0.f || !std::isfinite(desc->poisson) || desc->poisson < 0.f ||
        desc->poisson >= 0.5f || !std::isfinite(desc->strainDamping) || desc->strainDamping < 0.f) return -2004;
    int cc = desc->cornerCount, bpc = desc->bendPairCount;
    if (cc <= 0) return -2001;
    if (!S.reconReady || cc != S.N) return -2002;
    if (!mass || !pinned || !active || !extForce || !nbrIdx || !restNbr || (bpc > 0 && !bendPairs) || bpc < 0) return ERR_BAD_ARG;
    S.pd = *desc;
    S.mass.assign(mass, mass + cc);
    S.pinned.assign(pinned, pinned + cc); S.active.assign(active, active + cc);
    S.nbr.assign(nbrIdx, nbrIdx + (size_t)6 * cc);
    S.ext.resize(cc); S.vel.assign(cc, v3(0, 0, 0)); S.prev = S.pos;
    for (int i = 0; i < cc; i++) S.ext[i] = v3(extForce[3 * i], extForce[3 * i + 1], extForce[3 * i + 2]);
    S.bends.assign((const BendPair*)bendPairs, (const BendPair*)bendPairs + bpc);
    S.numSubsteps = desc->maxSubsteps > 0 ? desc->maxSubsteps : 20;
    S.omega = 1; S.damping = 0; S.ks = desc->ks; S.kb = desc->kb; S.alpha = desc->alpha; S.betaS = desc->cs; S.betaB = desc->cb;
    S.youngE = desc->youngE; S.poisson = desc->poisson; S.strainDamping = desc->strainDamping;

    // canonical edges from each node's positive slots (xpbd_solver.cu:1445-1463)
    std::vector<int> ends, own; std::vector<Real> rl;
    for (int p = 0; p < cc; p++)
        for (int a = 0; a < 3; a++) {
            int s = 2 * a + 1, n = S.nbr[(size_t)6 * p + s];
            if (n < 0) continue;
            if (n >= cc) return ERR_BAD_ARG;
            const float* r = restNbr + (size_t)3 * (6 * p + s);
            ends.push_back(p); ends.push_back(n); own.push_back(6 * p + s);
            if (sizeof(Real) == 4) rl.push_back((Real)std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]));
            else rl.push_back((Real)std::sqrt((double)r[0] * r[0] + (double)r[1] * r[1] + (double)r[2] * r[2]));
        }
    int E = (int)own.size(), nc = 0;
    std::vector<int> colour, slotOf;
    int rc = greedyColour<2>(E, ends.data(), cc, colour, nc);
    if (rc) return rc;
    bucket(colour, nc, S.eColOff, S.eColCnt, slotOf);
    S.E = E; S.eI.assign(E, 0); S.eJ.assign(E, 0); S.eOwner.assign(E, 0); S.eRest.assign(E, 0); S.eActive.assign(E, 1);
    for (int e = 0; e < E; e++) {
        int d = slotOf[e];
        S.eI[d] = ends[2 * e]; S.eJ[d] = ends[2 * e + 1]; S.eOwner[d] = own[e]; S.eRest[d] = rl[e];
    }
    // bend elements alive at bind time, colouring over their three nodes (xpbd_solver.cu:1465-1479, 1332-1400)
    std::vector<int> ijk, src; std::vector<Real> th;
    for (int b = 0; b < bpc; b++) {
        const BendPair& bp = S.bends[b];
        if (!bp.alive) continue;
        if (bp.i < 0 || bp.i >= cc || bp.j < 0 || bp.j >= cc || bp.k < 0 || bp.k >= cc) return ERR_BAD_ARG;
        ijk.push_back(bp.i); ijk.push_back(bp.j); ijk.push_back(bp.k); th.push_back(bp.theta0); src.push_back(b);
    }
    int B = (int)src.size();
    rc = greedyColour<3>(B, ijk.data(), cc, colour, nc);
    if (rc) return rc;
    bucket(colour, nc, S.bColOff, S.bColCnt, slotOf);
    S.B = B; S.bI.assign(B, 0); S.bJ.assign(B, 0); S.bK.assign(B, 0); S.bSrc.assign(B, 0); S.bTheta.assign(B, 0); S.bActive.assign(B, 1);
    for (int e = 0; e < B; e++) {
        int d = slotOf[e];
        S.bI[d] = ijk[3 * e]; S.bJ[d] = ijk[3 * e + 1]; S.bK[d] = ijk[3 * e + 2]; S.bTheta[d] = th[e]; S.bSrc[d] = src[e];
    }
    S.invMass.assign(cc, 0);
    for (int c = 0; c < cc; c++) S.invMass[c] = (S.pinned[c] || !S.active[c]) ? Real(0) : Real(1) / S.mass[c];
    S.jawLambda.assign(cc, 0); S.shaftLambda.assign(cc, 0);
    rc = buildTets();
    if (rc) return rc;
    resetParticleFrames();   // identity frames (V/physics.cu:258-267)
    S.physReady = true;
    S.livenessStale = true;
    return 0;
}

API int LCS_PhysicsAbiVersion() { return (int)sizeof(PhysicsInitDesc); }
API int LCS_GraspToolAbiVersion() { return (int)sizeof(XpbdToolState); }
API int LCS_ContactModelVersion() { return 28; }

API int LCS_SetGravity(float gx, float gy, float gz) {
    if (!S.physReady) return ERR_NOT_READY;
    if (!std::isfinite(gx) || !std::isfinite(gy) || !std::isfinite(gz)) return ERR_BAD_ARG;
    for (int i = 0; i < S.N; i++) S.ext[i] = v3((Real)gx * S.mass[i], (Real)gy * S.mass[i], (Real)gz * S.mass[i]);
    return 0;
}

// Per-tet material (extension): mu*V and kappa*V per tet in storage order; alpha = 1/(h^2 * stiffness).
API int LCS_SetTetStiffness(int count, const float* muV, const float* kappaV) {
    if (!S.physReady) return ERR_NOT_READY;
    if (count != S.T || !muV || !kappaV) return ERR_BAD_ARG;
    for (int t = 0; t < count; t++)
        if (!(muV[t] > 0.f) || !(kappaV[t] > 0.f) || !std::isfinite(muV[t]) || !std::isfinite(kappaV[t])) return ERR_BAD_ARG;
    for (int t = 0; t < count; t++) { S.muV[t] = muV[t]; S.kappaV[t] = kappaV[t]; }
    S.frameReady = false;
    return 0;
}
API int LCS_GetTetStiffness(float* muV, float* kappaV) {
    if (!S.physReady || !muV || !kappaV) return ERR_BAD_ARG;
    for (int t = 0; t < S.T; t++) { muV[t] = (float)S.muV[t]; kappaV[t] = (float)S.kappaV[t]; }
    return 0;
}
API int LCS_TetCount() { return S.physReady ? S.T : 0; }
API int LCS_TetColorCount() { return S.physReady ? (int)S.tColCnt.size() : 0; }
API int LCS_EdgeColorCount() { return S.physReady ? (int)S.eColCnt.size() : 0; }
API int LCS_EdgeCount() { return S.physReady ? S.E : 0; }
API int LCS_GetTetIds(int* out) {
    if (!S.physReady || !out) return ERR_BAD_ARG;
    std::memcpy(out, S.tIds.data(), S.tIds.size() * sizeof(int));
    return 0;
}
// colour of every tet in storage order / of every edge keyed by its owner slot (6p+s), -1 elsewhere
API int LCS_GetTetColors(int* out) {
    if (!S.physReady || !out) return ERR_BAD_ARG;
    for (size_t c = 0; c < S.tColCnt.size(); c++)
        for (int k = 0; k < S.tColCnt[c]; k++) out[S.tColorOrder[S.tColOff[c] + k]] = (int)c;
    return 0;
}
API int LCS_GetEdgeColors(int* out6N) {
    if (!S.physReady || !out6N) return ERR_BAD_ARG;
    for (int i = 0; i < 6 * S.N; i++) out6N[i] = -1;
    for (size_t c = 0; c < S.eColCnt.size(); c++)
        for (int k = 0; k < S.eColCnt[c]; k++) out6N[S.eOwner[S.eColOff[c] + k]] = (int)c;
    return 0;
}

// ---------------------------------------------------------------------------------------------
// contact model / grasp / guard setters (plain branch subset)
// ---------------------------------------------------------------------------------------------
API void LCS_SetGraspParams(const XpbdGraspParams* p) { if (p) S.gp = *p; }
API int LCS_SetContactModel(int enabled, float muS, float muD, float thickness, float radius) {
    if (!S.physReady) return ERR_NOT_READY;
    if (enabled < 0 || enabled > 2 || !std::isfinite(muS) || !std::isfinite(muD) || !std::isfinite(thickness) || !std::isfinite(radius) ||
        muS < 0 || muD < 0 || muD > muS || thickness <= 0 || radius < 0) return ERR_BAD_ARG;
    if (enabled == 2) return ERR_UNSUPPORTED;     // anchor assist belongs to the unified grasp solver
    S.contactModel = enabled; S.grasping = false;
    S.muStatic = muS; S.muDynamic = muD; S.jawThickness = thickness; S.contactRadius = radius;
    return 0;
}
// Tissue guard (xpbd_set_tissue_guard, xpbd_solver.cu:1892-1916): minimum relative volume and the
// number of tensile passes; passes > 0 also switches the tet projection to its guarded form and
// arms the feasibility chain.  `inside`/`capture` select grasp-capture wedges, which the plain
// branch never uses.
API int LCS_SetTissueGuard(float minimum, int passes, int count, const int* inside, int capture) {
    (void)capture;
    if (!S.physReady || S.h > 0 || !std::isfinite(minimum) || minimum < 0 || minimum > .95f || passes < 0 || passes > 4 || count != S.N || !inside)
        return ERR_BAD_ARG;
    // incident tets of every node, ascending tet index (storage order)
    S.incOff.assign(S.N + 1, 0);
    for (int t = 0; t < S.T; t++)
        for (int k = 0; k < 4; k++) S.incOff[S.tIds[4 * t + k] + 1]++;
    for (int i = 0; i < S.N; i++) S.incOff[i + 1] += S.incOff[i];
    S.incTet.assign((size_t)4 * S.T, 0);
    std::vector<int> cursor(S.incOff.begin(), S.incOff.end() - 1);
    for (int t = 0; t < S.T; t++)
        for (int k = 0; k < 4; k++) S.incTet[cursor[S.tIds[4 * t + k]]++] = t;
    S.needed.assign(S.N, 0);
    S.feasTarget.assign(S.N, v3(0, 0, 0));
    S.fiberLambda.assign((size_t)6 * S.T, Real(0));
    S.minVolume = (Real)minimum;
    S.volumePasses = passes;
    for (int k = 0; k < 3; k++) S.guardStats[k] = 0;
    return 0;
}
API int LCS_SetTissueMaterial(float strength, float bulkDamping) {
    if (!S.physReady || S.h > 0 || !std::isfinite(strength) || strength < 0 || strength > 1000 || !std::isfinite(bulkDamping) ||
        bulkDamping < 0 || bulkDamping > 1) return ERR_BAD_ARG;
    S.tissueHardening = strength; S.bulkDampingSeconds = bulkDamping;
    return 0;
}
API int LCS_SetGraspTool(const XpbdToolState* t) {
    if (!S.physReady || !t) return -1;
    S.toolFrom = S.toolArmed ? S.tool : *t;
    S.tool = *t; S.toolArmed = true;
    if (t->grasp01 > S.gp.graspThreshold) return ERR_UNSUPPORTED;   // capture starts the grasp path
    return 0;
}

// ---------------------------------------------------------------------------------------------
// frame + substep
// ---------------------------------------------------------------------------------------------
static int beginFrame(float dt) {
    S.frameReady = false;
    int N = S.numSubsteps > 0 ? S.numSubsteps : 1;
    Real h = (Real)dt / (Real)N;
    if (!(h > 0) || !isFin(h)) return ERR_BAD_DT;
    Real at = S.ks > 0 ? Real(1) / (S.ks * h * h) : Real(0);
    S.velScale = (Real(1) - S.damping) / (Real(1) + S.alpha * h);
    S.betaGammaHS = at * S.betaS * h;
    S.alphaTilde = at;
    S.doBend = S.B > 0 && S.kb > 0;
    S.alphaB = S.doBend ? Real(1) / (S.kb * h * h) : Real(0);
    S.betaGammaHB = S.alphaB * S.betaB * h;
    S.h = h;
    S.doStrain = S.T > 0 && S.youngE > 0;
    if (S.doStrain) {
        Real invH2 = Real(1) / (h * h);
        for (int t = 0; t < S.T; t++) { S.aDev[t] = invH2 / S.muV[t]; S.aHyd[t] = invH2 / S.kappaV[t]; }
    }
    S.substepIndex = 0;
    S.frameReady = true;
    return 0;
}

static void refreshLiveness() {
    if (!S.livenessStale && S.livenessRevision == S.revision) return;
    for (int e = 0; e < S.E; e++)
        S.eActive[e] = (S.nbr[S.eOwner[e]] >= 0 && S.active[S.eI[e]] && S.active[S.eJ[e]]) ? 1 : 0;
    for (int b = 0; b < S.B; b++) S.bActive[b] = S.bends[S.bSrc[b]].alive ? 1 : 0;
    for (int c = 0; c < S.N; c++) S.invMass[c] = (S.pinned[c] || !S.active[c]) ? Real(0) : Real(1) / S.mass[c];
    for (int t = 0; t < S.T; t++) {
        const int* o = &S.tOwner[3 * t]; const int* d = &S.tIds[4 * t];
        S.tActive[t] = (S.nbr[o[0]] >= 0 && S.nbr[o[1]] >= 0 && S.nbr[o[2]] >= 0 && S.active[d[0]] && S.active[d[1]] && S.active[d[2]] && S.active[d[3]]) ? 1 : 0;
    }
    std::fill(S.edgeSupport.begin(), S.edgeSupport.end(), 0);
    for (int t = 0; t < S.T; t++)
        if (S.tActive[t])
            for (int k = 0; k < 3; k++) S.edgeSupport[S.tOwner[3 * t + k]] = 1;
    S.livenessStale = false;
    S.livenessRevision = S.revision;
}

static void projectEdge(int e, Real alphaTilde, Real gamma, bool fallback, Real fallbackInvEh2) {
    if (!S.eActive[e]) return;
    if (fallback) {
        if (S.edgeSupport[S.eOwner[e]]) return;
        alphaTilde = fallbackInvEh2 / S.eRest[e];
    }
    int i = S.eI[e], j = S.eJ[e];
    Real wi = S.invMass[i], wj = S.invMass[j], ws = wi + wj;
    if (ws <= 0) return;
    V3 d = S.pos[i] - S.pos[j];
    Real L = std::sqrt(dotF(d, d));
    if (L < Real(1e-9)) return;
    V3 n = d * (Real(1) / L);
    Real C = L - S.eRest[e];
#ifdef ORACLE_AS_WRITTEN
    Real gradDx = dot(n, (S.pos[i] - S.prev[i]) - (S.pos[j] - S.prev[j]));
    Real dl = (-C - gamma * gradDx) / ((Real(1) + gamma) * ws + alphaTilde);
#else
    // the library's form: without edge damping (gamma = 0) the damping term is a zero and is not formed
    Real num = gamma != Real(0) ? fmaR(-gamma, dotF(n, (S.pos[i] - S.prev[i]) - (S.pos[j] - S.prev[j])), -C) : -C;
    Real dl = num / fmaR(Real(1) + gamma, ws, alphaTilde);
#endif
    Real ap = S.omega * dl;
    S.pos[i] = fmv(n, wi * ap, S.pos[i]);
    S.pos[j] = fmv(n, -(wj * ap), S.pos[j]);
}

static void projectBend(int e) {
    if (!S.bActive[e]) return;
    int i = S.bI[e], j = S.bJ[e], k = S.bK[e];
    Real wi = S.invMass[i], wj = S.invMass[j], wk = S.invMass[k];
    if (wi + wj + wk <= 0) return;
    V3 u = S.pos[i] - S.pos[j], v = S.pos[i] - S.pos[k];
    Real Lu = len(u), Lv = len(v);
    if (Lu < Real(1e-9) || Lv < Real(1e-9)) return;
    V3 nu = u * (Real(1) / Lu), nv = v * (Real(1) / Lv);
    Real c = std::fmax(Real(-1), std::fmin(Real(1), dot(nu, nv)));
    Real s = std::sqrt(std::fmax(Real(1) - c * c, Real(0)));
    if (s < Real(1e-4)) return;
#ifdef ORACLE_AS_WRITTEN
    Real C = std::acos(c) - S.bTheta[e];   // acosf (xpbd_solver.cu:553)
#else
    Real C = acosBend(c) - S.bTheta[e];
#endif
    V3 gj = nv - nu * c, gk = nu - nv * c, gi = (gj + gk) * Real(-1);
    Real wg = wi * dot(gi, gi) + wj * dot(gj, gj) + wk * dot(gk, gk);
    Real g = S.betaGammaHB;
    Real gdx = dot(gi, S.pos[i] - S.prev[i]) + dot(gj, S.pos[j] - S.prev[j]) + dot(gk, S.pos[k] - S.prev[k]);
    Real den = (Real(1) + g) * wg + S.alphaB;
    if (den < Real(1e-12)) return;
    Real ap = S.omega * ((-C - g * gdx) / den);
    S.pos[i] = S.pos[i] + gi * (wi * ap);
    S.pos[j] = S.pos[j] + gj * (wj * ap);
    S.pos[k] = S.pos[k] + gk * (wk * ap);
}

static void projectTet(int e, Real dampingOverH, Real bulkDampingOverH) {
    if (!S.tActive[e]) return;
    const int* id = &S.tIds[4 * e];
    V3 p[4] = {S.pos[id[0]], S.pos[id[1]], S.pos[id[2]], S.pos[id[3]]};
    const Real(*Bm)[3] = S.typeB[S.tType[e]];
    V3 br[3] = {v3(Bm[0][0], Bm[0][1], Bm[0][2]), v3(Bm[1][0], Bm[1][1], Bm[1][2]), v3(Bm[2][0], Bm[2][1], Bm[2][2])};
    V3 e1 = p[1] - p[0], e2 = p[2] - p[0], e3 = p[3] - p[0];
    V3 F[3];
    for (int c = 0; c < 3; c++) F[c] = fmv(e3, comp(br[2], c), fmv(e2, comp(br[1], c), e1 * comp(br[0], c)));
    Real I1 = dotF(F[0], F[0]) + dotF(F[1], F[1]) + dotF(F[2], F[2]);
    V3 cof[3] = {crossF(F[1], F[2]), crossF(F[2], F[0]), crossF(F[0], F[1])};
    Real ad = S.aDev[e], ah = S.aHyd[e];
    Real J = dotF(F[0], cof[0]), pJ = std::fmax(J, Real(0.05));
#ifdef ORACLE_AS_WRITTEN
    // the reference's own operations (xpbd_solver.cu:773, 781): the library power and logarithm
    Real iso = std::pow(pJ, Real(-2.f / 3.f));
#else
    Real iso = powMinusTwoThirds(pJ);
#endif
    Real q = std::fmax(fmaR(iso, I1, Real(-3)), Real(0));
    Real CD = std::sqrt(std::fmax(q, Real(1e-12)));
    Real devScale = Real(1) / CD;
    Real volGrad = J > Real(0.05) ? iso * I1 / (Real(3) * pJ) : Real(0);
    // guarded (tissue guard armed): logarithmic bulk strain with a linear floor below J = 0.05
    const bool guarded = S.volumePasses > 0;
#ifdef ORACLE_AS_WRITTEN
    Real CH = guarded ? std::log(pJ) + std::fmin(Real(0), (J - Real(0.05)) / Real(0.05)) : J - Real(1);
#else
    Real CH = guarded ? logPositive(pJ) + std::fmin(Real(0), (J - Real(0.05)) / Real(0.05)) : J - Real(1);
#endif
    V3 gd[4], gh[4];
    for (int k = 1; k < 4; k++) {
        V3 b = br[k - 1];
        gh[k] = fmv(cof[2], b.z, fmv(cof[1], b.y, cof[0] * b.x));
        gd[k] = fmv(fmv(F[2], b.z, fmv(F[1], b.y, F[0] * b.x)), iso, gh[k] * -volGrad) * devScale;
        if (guarded) gh[k] = gh[k] * (Real(1) / pJ);
    }
    gd[0] = (gd[1] + gd[2] + gd[3]) * Real(-1);
    gh[0] = (gh[1] + gh[2] + gh[3]) * Real(-1);
#ifdef ORACLE_AS_WRITTEN
    const bool damped = true;
#else
    // the library's form: without strain (or guarded bulk) damping vd, vh enter multiplied by zero
    // and are not formed
    const bool damped = dampingOverH != Real(0) || (guarded && bulkDampingOverH != Real(0));
#endif
    Real dd = 0, dh = 0, hh = 0, vd = 0, vh = 0, w[4];
    for (int k = 0; k < 4; k++) {
        w[k] = S.invMass[id[k]];
        dd = fmaR(w[k], dotF(gd[k], gd[k]), dd); dh = fmaR(w[k], dotF(gd[k], gh[k]), dh); hh += w[k] * dot(gh[k], gh[k]);
        if (damped) {
            V3 dx = p[k] - S.prev[id[k]];
            vd += dotF(gd[k], dx); vh += dotF(gh[k], dx);
        }
    }
    (void)hh;
    Real scale = Real(1) + dampingOverH, bulkScale = guarded ? Real(1) + bulkDampingOverH : scale;
#ifdef ORACLE_AS_WRITTEN
    // the reference's divisions as written (xpbd_solver.cu:805-816)
    Real eAd = ad / scale, eAh = ah / bulkScale;
    Real A = dd + eAd, Bc = dh, gamma = Bc / A;
    Real schur = eAh + eAd * gamma * gamma;
    for (int k = 0; k < 4; k++) { V3 r = gh[k] - gd[k] * gamma; schur += w[k] * dot(r, r); }
    Real rd = (-CD - dampingOverH * vd) / scale;
    Real rh = (-CH - (bulkScale - Real(1)) * vh) / bulkScale;
    if (!(A > 0) || !(schur > 0)) return;
    Real dlH = S.omega * (rh - gamma * rd) / schur, dlD = (S.omega * rd - Bc * dlH) / A;
#else
    // the frame constant 1 / (1 + D/h) and one reciprocal of A (the library's form of the solve)
    Real invScale = Real(1) / scale, invBulk = Real(1) / bulkScale;
    Real eAd = ad * invScale, eAh = ah * invBulk;
    Real A = dd + eAd, invA = Real(1) / A, Bc = dh, gamma = Bc * invA;
    Real schur = fmaR(eAd * gamma, gamma, eAh);
    for (int k = 0; k < 4; k++) { V3 r = fmv(gd[k], -gamma, gh[k]); schur = fmaR(w[k], dotF(r, r), schur); }
    Real rd = damped ? fmaR(-dampingOverH, vd, -CD) * invScale : -CD * invScale;
    Real rh = damped ? fmaR(-(bulkScale - Real(1)), vh, -CH) * invBulk : -CH * invBulk;
    if (!(A > 0) || !(schur > 0)) return;
    Real dlH = S.omega * fmaR(-gamma, rd, rh) / schur, dlD = fmaR(-Bc, dlH, S.omega * rd) * invA;
#endif
    if (!isFin(dlD) || !isFin(dlH)) return;
    if (guarded) {   // trust region on the update: no corner moves more than 0.15 of the shortest rest edge scale
        Real largest = 0;
        for (int k = 0; k < 4; k++) largest = std::fmax(largest, len(fmv(gd[k], dlD, gh[k] * dlH) * w[k]));
        Real limit = Real(0.15) / std::fmax(len(br[0]), std::fmax(len(br[1]), len(br[2])));
        Real accepted = largest > limit ? limit / largest : Real(1);
        dlD *= accepted; dlH *= accepted;
    }
    for (int k = 0; k < 4; k++) S.pos[id[k]] = fmv(fmv(gd[k], dlD, gh[k] * dlH), w[k], p[k]);
}

// Tensile reinforcement of one live tet (projectTensile, xpbd_solver.cu:592-620): each of the six
// corner-to-corner fibres carries the energy mu V strength / 2 s^6, s = max(length / rest - 1, 0),
// projected with finite compliance alphaDev / strength; the rest corners are the columns of the
// inverse of the rest matrix Dm^-1.  `pass` > 0 continues the fibres' multipliers of this substep.
static void projectTensile(int e, int pass) {
    if (!S.tActive[e]) return;
    const Real strength = (Real)S.tissueHardening;
    if (!(strength > 0)) return;
    const int* id = &S.tIds[4 * e];
    V3 p[4] = {S.pos[id[0]], S.pos[id[1]], S.pos[id[2]], S.pos[id[3]]};
    const Real(*Bm)[3] = S.typeB[S.tType[e]];
    V3 b[3] = {v3(Bm[0][0], Bm[0][1], Bm[0][2]), v3(Bm[1][0], Bm[1][1], Bm[1][2]), v3(Bm[2][0], Bm[2][1], Bm[2][2])};
    Real detB = dot(b[0], cross(b[1], b[2]));
    V3 rest[4] = {v3(0, 0, 0), cross(b[1], b[2]) * (Real(1) / detB), cross(b[2], b[0]) * (Real(1) / detB), cross(b[0], b[1]) * (Real(1) / detB)};
    int fiber = 0;
    for (int i = 0; i < 4; i++)
        for (int k = i + 1; k < 4; k++, fiber++) {
            V3 edge = p[k] - p[i];
            Real length = len(edge), restLength = len(rest[k] - rest[i]);
            Real strain = std::fmax(length / restLength - Real(1), Real(0)), gradient = Real(3) * strain * strain / restLength;
            Real wi = S.invMass[id[i]], wk = S.invMass[id[k]], alpha = S.aDev[e] / std::fmax(strength, Real(1e-10));
            Real& lambda = S.fiberLambda[6 * (size_t)e + fiber];
            if (pass == 0) lambda = 0;
            if (strain > 0 && length > 0) {
                Real dl = (-strain * strain * strain - alpha * lambda) / ((wi + wk) * gradient * gradient + alpha);
                V3 g = edge * (gradient / length);
                lambda += dl;
                p[i] = p[i] - g * (wi * dl);
                p[k] = p[k] + g * (wk * dl);
            }
        }
    for (int k = 0; k < 4; k++) S.pos[id[k]] = p[k];
}

// Relative volume det(Ds) det(Dm^-1) of a tet from the given positions (storage order).
static Real tetVolume(int t, const std::vector<V3>& x) {
    const int* id = &S.tIds[4 * t];
    const Real(*Bm)[3] = S.typeB[S.tType[t]];
    V3 b0 = v3(Bm[0][0], Bm[0][1], Bm[0][2]), b1 = v3(Bm[1][0], Bm[1][1], Bm[1][2]), b2 = v3(Bm[2][0], Bm[2][1], Bm[2][2]);
    V3 a = x[id[0]], u = x[id[1]] - a, v = x[id[2]] - a, w = x[id[3]] - a;
    return dot(u, cross(v, w)) * dot(b0, cross(b1, b2));
}

// The feasibility chain of a guarded substep (finishFeasible, xpbd_solver.cu:628-741), after contact:
// if a live tet is below the minimum relative volume, two colour sweeps of a linearised volume repair;
// if one still is, every vertex of a tet whose motion over the substep may pass below the minimum
// (a conservative bound, then the 16 corners of the multi-affine volume) restarts from its
// substep-start position and advances along its candidate displacement as far as every incident
// live tet allows, in eight lattice-parity colours whose order rotates with the substep.
static void finishFeasible(int substepIndex) {
    const Real minimum = S.minVolume;
    bool unsafe = false;
    for (int t = 0; t < S.T && !unsafe; t++) {
        if (!S.tActive[t]) continue;
        Real J = tetVolume(t, S.pos);
        if (!isFin(J) || J < minimum) unsafe = true;
    }
    if (!unsafe) return;
    S.guardStats[0]++;
    for (int pass = 0; pass < 2; pass++)
        for (size_t c = 0; c < S.tColCnt.size(); c++) {
            int off = S.tColOff[c], cnt = S.tColCnt[c];
#pragma omp parallel for schedule(static)
            for (int k = 0; k < cnt; k++) {
                int t = S.tColorOrder[off + k];
                if (!S.tActive[t]) continue;
                const int* id = &S.tIds[4 * t];
                const Real(*Bm)[3] = S.typeB[S.tType[t]];
                V3 b0 = v3(Bm[0][0], Bm[0][1], Bm[0][2]), b1 = v3(Bm[1][0], Bm[1][1], Bm[1][2]), b2 = v3(Bm[2][0], Bm[2][1], Bm[2][2]);
                V3 p[4] = {S.pos[id[0]], S.pos[id[1]], S.pos[id[2]], S.pos[id[3]]};
                V3 u = p[1] - p[0], v = p[2] - p[0], w = p[3] - p[0];
                Real detB = dot(b0, cross(b1, b2));
                Real J = dot(u, cross(v, w)) * detB;
                if (!isFin(J) || J >= minimum + Real(1e-4)) continue;
                V3 g[4];
                g[1] = cross(v, w) * detB; g[2] = cross(w, u) * detB; g[3] = cross(u, v) * detB;
                g[0] = (g[1] + g[2] + g[3]) * Real(-1);
                Real den = 0;
                for (int n = 0; n < 4; n++) den += S.invMass[id[n]] * dot(g[n], g[n]);
                if (den < Real(1e-20)) continue;
                Real dl = (minimum + Real(2e-4) - J) / den;
                for (int n = 0; n < 4; n++) S.pos[id[n]] = p[n] + g[n] * (S.invMass[id[n]] * dl);
            }
        }
    unsafe = false;
    for (int t = 0; t < S.T && !unsafe; t++) {
        if (!S.tActive[t]) continue;
        Real J = tetVolume(t, S.pos);
        if (!isFin(J) || J < minimum) unsafe = true;
    }
    if (!unsafe) return;
    S.guardStats[1]++;
    std::fill(S.needed.begin(), S.needed.end(), 0);
    for (int t = 0; t < S.T; t++) {
        if (!S.tActive[t]) continue;
        const int* id = &S.tIds[4 * t];
        const Real(*Bm)[3] = S.typeB[S.tType[t]];
        V3 b0 = v3(Bm[0][0], Bm[0][1], Bm[0][2]), b1 = v3(Bm[1][0], Bm[1][1], Bm[1][2]), b2 = v3(Bm[2][0], Bm[2][1], Bm[2][2]);
        V3 x[4], d[4];
        for (int k = 0; k < 4; k++) { x[k] = S.prev[id[k]]; d[k] = S.pos[id[k]] - x[k]; }
        Real detB = dot(b0, cross(b1, b2));
        V3 u = x[1] - x[0], vv = x[2] - x[0], w = x[3] - x[0];
        Real r0 = len(d[0]), r1 = r0 + len(d[1]), r2 = r0 + len(d[2]), r3 = r0 + len(d[3]);
        Real bound = r1 * len(cross(vv, w)) + r2 * len(cross(w, u)) + r3 * len(cross(u, vv)) + r1 * r2 * len(w) + r1 * r3 * len(vv) +
                     r2 * r3 * len(u) + r1 * r2 * r3;
        if (dot(u, cross(vv, w)) * detB - bound * std::fabs(detB) >= minimum + Real(1e-5)) continue;
        bool bad = false;
        for (int mask = 0; mask < 16 && !bad; mask++) {
            V3 p[4];
            for (int k = 0; k < 4; k++) p[k] = x[k] + d[k] * (Real)((mask >> k) & 1);
            Real j = dot(p[1] - p[0], cross(p[2] - p[0], p[3] - p[0])) * detB;
            if (!isFin(j) || j < minimum + Real(1e-5)) bad = true;
        }
        if (bad)
            for (int k = 0; k < 4; k++) S.needed[id[k]] = 1;
    }
    for (int i = 0; i < S.N; i++)
        if (S.needed[i]) { S.feasTarget[i] = S.pos[i]; S.pos[i] = S.prev[i]; S.guardStats[2]++; }
    const int nx = S.dx + 1, ny = S.dy + 1, nz = S.dz + 1, phase = substepIndex & 7;
    for (int k = 0; k < 8; k++) {
        int color = (k + phase) & 7;
#pragma omp parallel for schedule(static)
        for (int z = (color >> 2) & 1; z < nz; z += 2)
            for (int y = (color >> 1) & 1; y < ny; y += 2)
                for (int x0 = color & 1; x0 < nx; x0 += 2) {
                    int i = x0 + nx * (y + ny * z);
                    if (!S.needed[i]) continue;
                    V3 delta = S.feasTarget[i] - S.pos[i];
                    Real accepted = 1;
                    if (!isFin(delta.x + delta.y + delta.z)) continue;
                    for (int q = S.incOff[i]; q < S.incOff[i + 1]; q++) {
                        int t = S.incTet[q];
                        if (!S.tActive[t]) continue;
                        const int* id = &S.tIds[4 * t];
                        const Real(*Bm)[3] = S.typeB[S.tType[t]];
                        V3 b0 = v3(Bm[0][0], Bm[0][1], Bm[0][2]), b1 = v3(Bm[1][0], Bm[1][1], Bm[1][2]), b2 = v3(Bm[2][0], Bm[2][1], Bm[2][2]);
                        V3 a = S.pos[id[0]], u = S.pos[id[1]] - a, v = S.pos[id[2]] - a, w = S.pos[id[3]] - a;
                        Real detB = dot(b0, cross(b1, b2));
                        Real j = dot(u, cross(v, w)) * detB;
                        V3 grad[3] = {cross(v, w), cross(w, u), cross(u, v)};
                        V3 g = i == id[0] ? (grad[0] + grad[1] + grad[2]) * Real(-1) : i == id[1] ? grad[0] : i == id[2] ? grad[1] : grad[2];
                        Real dj = dot(g, delta) * detB;
                        if (dj < 0) {
                            Real floor = std::fmin(minimum, std::fmax(Real(0), j));
                            if (j + dj < floor) accepted = std::fmin(accepted, std::fmax(Real(0), Real(0.95) * (j - floor) / (-dj)));
                        }
                    }
                    S.pos[i] = S.pos[i] + delta * accepted;
                }
    }
}

static V3 lerpF(const F3& a, const F3& b, Real t) { return fromF(a) * (Real(1) - t) + fromF(b) * t; }

static void solveContact(const V3& shaftA, const V3& shaftB, Real shaftR, const V3& hinge, const V3& axis, const V3& normal, const V3& w,
                         Real jawLen, Real jawHalfWidth, Real gapHalf, Real contactAlpha) {
    const Real omega = S.gp.ccdOmega, thresh = S.gp.ccdVelThresh, maxDisp = S.gp.ccdMaxDisp;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < S.N; c++) {
        Real wc = S.invMass[c];
        if (wc <= 0) continue;
        {
            V3 ab = shaftB - shaftA;
            Real ab2 = dot(ab, ab);
            Real tt = ab2 > Real(1e-12) ? dot(S.pos[c] - shaftA, ab) / ab2 : Real(0);
            tt = std::fmax(Real(0), std::fmin(Real(1), tt));
            V3 cl = shaftA + ab * tt, dv = S.pos[c] - cl;
            Real dist = len(dv), C = dist - shaftR;
            if (C < 0) {
                V3 n = dist > Real(1e-9) ? dv * (Real(1) / dist) : v3(0, 1, 0);
                if (-dot(S.vel[c], n) > thresh) {
                    Real dl = (-C - contactAlpha * S.shaftLambda[c]) / (wc + contactAlpha);
                    Real ap = omega * dl;
                    V3 corr = n * (wc * ap);
                    Real cl2 = len(corr);
                    if (cl2 > maxDisp) { Real s = maxDisp / cl2; ap *= s; corr = corr * s; }
                    S.shaftLambda[c] += ap;
                    S.pos[c] = S.pos[c] + corr;
                }
            }
        }
        {   // jaw slab box (no capture happens on this path, so no node is grasped)
            V3 rel = S.pos[c] - hinge;
            Real u = dot(rel, axis), v = dot(rel, w), n = dot(rel, normal);
            if (u >= 0 && u <= jawLen && std::fabs(v) <= jawHalfWidth) {
                Real an = std::fabs(n);
                if (an > gapHalf) {
                    Real C = gapHalf - an, sg = n >= 0 ? Real(1) : Real(-1);
                    V3 nOut = normal * sg;
                    if (-dot(S.vel[c], nOut) > thresh) {
                        Real dl = (-C - contactAlpha * S.jawLambda[c]) / (wc + contactAlpha);
                        Real ap = omega * dl, cm = wc * ap;
                        if (std::fabs(cm) > maxDisp) { Real s = maxDisp / std::fabs(cm); ap *= s; cm *= s; }
                        S.jawLambda[c] += ap;
                        S.pos[c] = S.pos[c] - normal * (sg * cm);
                    }
                }
            }
        }
    }
}

#include "friction_oracle.inc"

static int substep() {
    if (!S.physReady) return ERR_NOT_READY;
    if (!S.frameReady) return ERR_NO_FRAME;
    const Real h = S.h;
    const int NS = S.numSubsteps > 0 ? S.numSubsteps : 1;
    Real t = std::min(Real(1), Real(++S.substepIndex) / Real(NS));
    refreshLiveness();
    const bool fallback = S.doStrain && S.ks <= 0;
    // predict
#pragma omp parallel for schedule(static)
    for (int p = 0; p < S.N; p++) {
        S.prev[p] = S.pos[p];
        if (S.invMass[p] > 0) {
            V3 a = S.ext[p] * S.invMass[p];
            V3 v = S.vel[p] + a * h;
            S.vel[p] = v;
            S.pos[p] = S.pos[p] + v * h;
        }
    }
    if (S.ks > 0 || fallback) {
        Real fb = fallback ? Real(1) / (S.youngE * h * h) : Real(0);
        for (size_t c = 0; c < S.eColCnt.size(); c++) {
            int off = S.eColOff[c], cnt = S.eColCnt[c];
#pragma omp parallel for schedule(static)
            for (int k = 0; k < cnt; k++) projectEdge(off + k, S.alphaTilde, S.betaGammaHS, fallback, fb);
        }
    }
    if (S.doBend)
        for (size_t c = 0; c < S.bColCnt.size(); c++) {
            int off = S.bColOff[c], cnt = S.bColCnt[c];
#pragma omp parallel for schedule(static)
            for (int k = 0; k < cnt; k++) projectBend(off + k);
        }
    if (S.doStrain) {
        Real dOH = std::fmax(Real(0), S.strainDamping) / h;
        Real bOH = h > 0 ? Real(S.bulkDampingSeconds) / h : Real(0);
        for (size_t c = 0; c < S.tColCnt.size(); c++) {
            int off = S.tColOff[c], cnt = S.tColCnt[c];
#pragma omp parallel for schedule(static)
            for (int k = 0; k < cnt; k++) projectTet(S.tColorOrder[off + k], dOH, bOH);
        }
        for (int pass = 0; pass < S.volumePasses; pass++)   // tensile reinforcement (solveTetGraph, xpbd_solver.cu:2531-2533)
            for (size_t c = 0; c < S.tColCnt.size(); c++) {
                int off = S.tColOff[c], cnt = S.tColCnt[c];
#pragma omp parallel for schedule(static)
                for (int k = 0; k < cnt; k++) projectTensile(S.tColorOrder[off + k], pass);
            }
    }
    if (S.toolArmed && S.contactModel == 0) {
        std::fill(S.jawLambda.begin(), S.jawLambda.end(), Real(0));
        std::fill(S.shaftLambda.begin(), S.shaftLambda.end(), Real(0));
        XpbdToolState st = S.tool;
        V3 hinge = lerpF(S.toolFrom.jawHinge, S.tool.jawHinge, t);
        V3 ax = lerpF(S.toolFrom.jawAxis, S.tool.jawAxis, t);
        V3 nm = lerpF(S.toolFrom.jawNormal, S.tool.jawNormal, t);
        V3 sa = lerpF(S.toolFrom.shaftA, S.tool.shaftA, t), sb = lerpF(S.toolFrom.shaftB, S.tool.shaftB, t);
        Real gap = (Real)S.toolFrom.jawGap * (Real(1) - t) + (Real)S.tool.jawGap * t;
        V3 axis = len(ax) > Real(1e-9) ? ax * (Real(1) / len(ax)) : v3(0, 0, 1);
        V3 normal = len(nm) > Real(1e-9) ? nm * (Real(1) / len(nm)) : v3(0, 1, 0);
        normal = normal - axis * dot(normal, axis);
        if (len(normal) < Real(1e-7)) normal = cross(axis, std::fabs(axis.x) < Real(0.9) ? v3(1, 0, 0) : v3(0, 1, 0));
        normal = normal * (Real(1) / len(normal));
        V3 w = cross(axis, normal);
        Real gapHalf = Real(0.5) * std::fmax(gap, (Real)S.gp.jawGapClosed);
        solveContact(sa, sb, st.shaftR, hinge, axis, normal, w, st.jawLen, st.jawHalfWidth, gapHalf, (Real)S.gp.contactAlpha / (h * h));
    }
    if (S.toolArmed && S.contactModel == 1) frictionContact(t);   // contact model 1, no surface (xpbd_solver.cu:3655-3665)
    if (S.volumePasses > 0 && S.T > 0) finishFeasible(S.substepIndex);
    Real invH = Real(1) / h;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < S.N; p++) S.vel[p] = S.invMass[p] > 0 ? (S.pos[p] - S.prev[p]) * invH : v3(0, 0, 0);
    if (S.betaS > 0)
        for (size_t c = 0; c < S.eColCnt.size(); c++) {
            int off = S.eColOff[c], cnt = S.eColCnt[c];
#pragma omp parallel for schedule(static)
            for (int k = 0; k < cnt; k++) {
                int e = off + k;
                if (!S.eActive[e]) continue;
                int i = S.eI[e], j = S.eJ[e];
                Real wi = S.invMass[i], wj = S.invMass[j];
                if (wi + wj <= 0) continue;
                V3 d = S.pos[i] - S.pos[j];
                Real L = len(d);
                if (L < Real(1e-9)) continue;
                V3 n = d * (Real(1) / L), vr = S.vel[i] - S.vel[j];
                V3 imp = (vr - n * dot(vr, n)) * (h * S.betaS);
                if (wi > 0) S.vel[i] = S.vel[i] - imp * wi;
                if (wj > 0) S.vel[j] = S.vel[j] + imp * wj;
            }
        }
#pragma omp parallel for schedule(static)
    for (int p = 0; p < S.N; p++) S.vel[p] = S.invMass[p] > 0 ? S.vel[p] * S.velScale : v3(0, 0, 0);
    if (S.substepIndex >= NS) S.toolFrom = S.tool;
    return 0;
}

// ---------------------------------------------------------------------------------------------
// cut: lattice edge stencil, Moller-Trumbore, mark, CCD, tear, sever
// ---------------------------------------------------------------------------------------------
static const int ES_OFF[3][4][3] = {{{0, 0, 0}, {0, -1, 0}, {0, -1, -1}, {0, 0, -1}},
                                    {{0, 0, 0}, {0, 0, -1}, {-1, 0, -1}, {-1, 0, 0}},
                                    {{0, 0, 0}, {-1, 0, 0}, {-1, -1, 0}, {0, -1, 0}}};
static const int ES_EDGE[3][4] = {{0, 2, 6, 4}, {3, 7, 5, 1}, {8, 9, 10, 11}};
static bool voxIn(int x, int y, int z) { return x >= 0 && y >= 0 && z >= 0 && x < S.dx && y < S.dy && z < S.dz; }
static int voxId(int x, int y, int z) { return x + S.dx * (y + S.dy * z); }
static bool edgeIsCut(const GridEdge2& g) {
    for (int s = 0; s < 4; s++) {
        int x = g.bx + ES_OFF[g.axis][s][0], y = g.by + ES_OFF[g.axis][s][1], z = g.bz + ES_OFF[g.axis][s][2];
        if (voxIn(x, y, z) && (S.cutMask[voxId(x, y, z)] >> ES_EDGE[g.axis][s] & 1u)) return true;
    }
    return false;
}
static bool edgeValid(const GridEdge2& g) {
    for (int s = 0; s < 4; s++)
        if (!voxIn(g.bx + ES_OFF[g.axis][s][0], g.by + ES_OFF[g.axis][s][1], g.bz + ES_OFF[g.axis][s][2])) return false;
    return true;
}
static bool cutHitsMaterial(float t, float skin, int ia, int ib) {
    if (ia && ib) return true;
    if (!ia && !ib) return false;
    if (!(skin >= 0.f && skin <= 1.f)) return false;
    return ia ? t <= skin : t >= skin;
}
// EmitCutPoint (V/cut.cu:186-215): owner p's cut point on the undeformed edge plus the half-kerf on
// its side of the cut plane, and the outward cut normal, both in p's current frame; stored at p's
// directed lattice slot (each lattice edge is first cut once, so a slot is written once).
static void emitCutPointO(int p, int slot, V3 hit, V3 along, V3 ncut) {
    const Real sd = dot(S.pos[p] - hit, ncut);
    Real side = sd > 0 ? Real(1) : (sd < 0 ? Real(-1) : Real(0));
    if (side == 0) side = 1;
    const Real* q = &S.particleRot[(size_t)9 * p];
    const V3 r0 = v3(q[0], q[1], q[2]), r1 = v3(q[3], q[4], q[5]), r2 = v3(q[6], q[7], q[8]);
    const V3 g = ncut * (side * (Real(S.cutTool.d) * Real(0.5f))), n = ncut * side;
    const V3 local = along + ((r0 * g.x + r1 * g.y) + r2 * g.z);
    const V3 mat = (r0 * n.x + r1 * n.y) + r2 * n.z;
    Real* rec = &S.cutRec[(size_t)8 * slot];
    rec[0] = local.x; rec[1] = local.y; rec[2] = local.z; rec[3] = 1;
    rec[4] = mat.x; rec[5] = mat.y; rec[6] = mat.z; rec[7] = 0;
}

static void markAndEmit(const GridEdge2& g, int idA, int idB, float tRay, V3 hit, V3 ncut) {
    bool first = false, saw = false, occ = false;
    for (int s = 0; s < 4; s++) {
        int x = g.bx + ES_OFF[g.axis][s][0], y = g.by + ES_OFF[g.axis][s][1], z = g.bz + ES_OFF[g.axis][s][2];
        if (!voxIn(x, y, z)) continue;
        int v = voxId(x, y, z);
        if (!S.occupied[v]) continue;
        occ = true;
        unsigned bit = 1u << ES_EDGE[g.axis][s], old = S.cutMask[v];
        S.cutMask[v] = old | bit;
        if (!saw) { saw = true; first = (old & bit) == 0; }
    }
    if (!(first && occ)) return;
    S.edgeCutT[slotOfDirected(idA, idB)] = tRay;
    S.edgeCutT[slotOfDirected(idB, idA)] = 1.f - tRay;
    if (!cutHitsMaterial(tRay, S.skinT[slotOfDirected(idA, idB)], S.inside[idA], S.inside[idB])) return;
    S.cutPoints += 2;
    const V3 rest = S.rest[idB] - S.rest[idA];
    emitCutPointO(idA, 6 * idA + 2 * g.axis + 1, hit, rest * Real(tRay), ncut);
    emitCutPointO(idB, 6 * idB + 2 * g.axis, hit, rest * (Real(tRay) - Real(1)), ncut);
}
static bool mollerTrumbore(V3 O, V3 D, V3 V0, V3 V1, V3 V2, Real& t, Real& u, Real& v) {
    V3 L1 = V1 - V0, L2 = V2 - V0, Tv = V0 - O;
    Real det = dot(cross(L2, D), L1);
    t = u = v = 0;
    if (std::fabs(det) < Real(1e-12)) return false;
    Real inv = Real(1) / det;
    t = dot(cross(L2, Tv), L1) * inv;
    u = -dot(cross(L2, D), Tv) * inv;
    v = dot(cross(D, Tv), L1) * inv;
    const Real EPS = Real(1e-5);
    return u >= -EPS && v >= -EPS && u + v <= Real(1) + EPS && t > 0 && t <= Real(1);
}
static void severLinks() {
    for (size_t e = 0; e < S.gridEdges.size(); e++) {
        const GridEdge2& g = S.gridEdges[e];
        if (!edgeValid(g) || !edgeIsCut(g)) continue;
        int a = cid(g.bx, g.by, g.bz), b = cid(g.bx + (g.axis == 0), g.by + (g.axis == 1), g.bz + (g.axis == 2));
        int ax = g.axis;
        if (S.nbr[6 * a + 2 * ax + 1] >= 0) S.revision++;
        S.nbr[6 * a + 2 * ax + 1] = -1;
        S.nbr[6 * b + 2 * ax] = -1;
        if ((size_t)15 * (std::max(a, b) + 1) > S.bends.size()) continue;
        for (int p = 0; p < 15; p++) {
            BendPair& x = S.bends[15 * a + p];
            if (x.alive && (x.j == b || x.k == b)) x.alive = 0;
            BendPair& y = S.bends[15 * b + p];
            if (y.alive && (y.j == a || y.k == a)) y.alive = 0;
        }
    }
}

API int LCS_InitCut(const CutInitDesc* desc, const void* conn4096, const void* gridEdges, const int* voxelOccupied, const int* cornerInside) {
    resetCut();
    if (!desc) return -3000;
    if (desc->voxelCount <= 0 || desc->cornerCount <= 0) return -3001;
    if (!S.physReady || desc->cornerCount != S.N || desc->dimsX != S.dx || desc->dimsY != S.dy || desc->dimsZ != S.dz) return -3002;
    if (desc->voxelCount != S.dx * S.dy * S.dz || !voxelOccupied || !cornerInside || (desc->gridEdgeCount > 0 && !gridEdges)) return -3001;
    S.cd = *desc;
    S.gridEdges.assign((const GridEdge2*)gridEdges, (const GridEdge2*)gridEdges + std::max(0, desc->gridEdgeCount));
    S.occupied.assign(voxelOccupied, voxelOccupied + desc->voxelCount);
    S.cutMask.assign(desc->voxelCount, 0u);
    S.inside.assign(cornerInside, cornerInside + S.N);
    S.edgeCutT.assign((size_t)6 * S.N, -1.f);
    S.prevCorner = S.pos;
    S.edgeWasExempt.assign(S.gridEdges.size(), 0); S.edgeDecay.assign(S.gridEdges.size(), 0);
    S.emitNcut = v3(0, 1, 0);
    S.cutRec.assign((size_t)48 * S.N, Real(0));
    S.conn.clear();
    if (conn4096) S.conn.assign((const int*)conn4096, (const int*)conn4096 + 9 * 4096);
    float tau = desc->tearStretchRatio;
    S.tearLen2 = (tau >= 1.0f && tau == tau) ? (Real)((tau * desc->voxelL) * (tau * desc->voxelL)) : Real(0);
    S.cutReady = true;
    return 0;
}
API void LCS_SetTool(const CutToolDesc* t) {
    if (!t) return;
    S.cutTool = *t;
    if (t->valid) S.emitNcut = fromA(t->ncut);
    if (!S.toolSet && S.cutReady) { S.prevCorner = S.pos; S.havePrev = true; }
    S.toolSet = true;
}
API void LCS_SetPressureCutMode(int enabled) { S.pressure = enabled != 0; }

API int LCS_DetectCut() {
    if (!S.cutReady || !S.toolSet || S.pressure) return 0;
    const CutToolDesc& c = S.cutTool;
    if (c.valid) {
        Real pad = S.cd.voxelL;
        V3 lo = fromA(c.aabbMin), hi = fromA(c.aabbMax);
        for (size_t e = 0; e < S.gridEdges.size(); e++) {
            const GridEdge2& g = S.gridEdges[e];
            int a = cid(g.bx, g.by, g.bz), b = cid(g.bx + (g.axis == 0), g.by + (g.axis == 1), g.bz + (g.axis == 2));
            V3 O = S.pos[a], D = S.pos[b] - O;
            V3 mn = v3(std::fmin(O.x, O.x + D.x), std::fmin(O.y, O.y + D.y), std::fmin(O.z, O.z + D.z));
            V3 mx = v3(std::fmax(O.x, O.x + D.x), std::fmax(O.y, O.y + D.y), std::fmax(O.z, O.z + D.z));
            if (mx.x < lo.x - pad || mn.x > hi.x + pad || mx.y < lo.y - pad || mn.y > hi.y + pad || mx.z < lo.z - pad || mn.z > hi.z + pad) continue;
            Real t1, u1, v1, t2, u2, v2;
            bool h1 = mollerTrumbore(O, D, fromA(c.t1v0), fromA(c.t1v1), fromA(c.t1v2), t1, u1, v1);
            bool h2 = mollerTrumbore(O, D, fromA(c.t2v0), fromA(c.t2v1), fromA(c.t2v2), t2, u2, v2);
            if (!h1 && !h2) continue;
            Real tr = (h1 && h2) ? std::fmin(t1, t2) : (h1 ? t1 : t2);
            tr = std::fmin(std::fmax(tr, Real(0)), Real(1));
            markAndEmit(g, a, b, (float)tr, O + D * tr, fromA(c.ncut));
        }
    }
    severLinks();
    return 0;
}

static int ribbonTick() {
    if (!S.cutReady || !S.toolSet || S.pressure) return 0;
    if (!S.havePrev) { S.prevCorner = S.pos; S.havePrev = true; return 0; }
    V3 Sg = fromA(S.cutTool.t2v2), Eg = fromA(S.cutTool.t1v2);
    Real pad = S.cd.voxelL;
    for (size_t e = 0; e < S.gridEdges.size(); e++) {
        const GridEdge2& g = S.gridEdges[e];
        int a = cid(g.bx, g.by, g.bz), b = cid(g.bx + (g.axis == 0), g.by + (g.axis == 1), g.bz + (g.axis == 2));
        if (S.nbr[6 * a + 2 * g.axis + 1] < 0) continue;
        V3 a0 = S.prevCorner[a], a1 = S.pos[a], b0 = S.prevCorner[b], b1 = S.pos[b];
        V3 sMin = v3(std::fmin(Sg.x, Eg.x) - pad, std::fmin(Sg.y, Eg.y) - pad, std::fmin(Sg.z, Eg.z) - pad);
        V3 sMax = v3(std::fmax(Sg.x, Eg.x) + pad, std::fmax(Sg.y, Eg.y) + pad, std::fmax(Sg.z, Eg.z) + pad);
        V3 eMin = v3(std::fmin(std::fmin(a0.x, a1.x), std::fmin(b0.x, b1.x)), std::fmin(std::fmin(a0.y, a1.y), std::fmin(b0.y, b1.y)),
                     std::fmin(std::fmin(a0.z, a1.z), std::fmin(b0.z, b1.z)));
        V3 eMax = v3(std::fmax(std::fmax(a0.x, a1.x), std::fmax(b0.x, b1.x)), std::fmax(std::fmax(a0.y, a1.y), std::fmax(b0.y, b1.y)),
                     std::fmax(std::fmax(a0.z, a1.z), std::fmax(b0.z, b1.z)));
        if (eMax.x < sMin.x || eMin.x > sMax.x || eMax.y < sMin.y || eMin.y > sMax.y || eMax.z < sMin.z || eMin.z > sMax.z) continue;
        V3 D = Eg - Sg, P0 = a0 - Sg, Pv = a1 - a0, Q0 = b0 - Sg, Qv = b1 - b0;
        Real c0 = dot(cross(P0, Q0), D), c1 = dot(cross(P0, Qv) + cross(Pv, Q0), D), c2 = dot(cross(Pv, Qv), D);
        Real roots[2]; int nr = 0;
        if (std::fabs(c2) < Real(1e-14)) {
            if (std::fabs(c1) > Real(1e-14)) { Real r = -c0 / c1; if (r >= 0 && r <= 1) roots[nr++] = r; }
        } else {
            Real disc = c1 * c1 - Real(4) * c2 * c0;
            if (disc >= 0) {
                Real sq = std::sqrt(disc), qq = Real(-0.5) * (c1 + (c1 >= 0 ? sq : -sq));
                Real r0 = qq / c2, r1 = std::fabs(qq) > Real(1e-20) ? c0 / qq : r0;
                if (r0 > r1) std::swap(r0, r1);
                if (r0 >= 0 && r0 <= 1) roots[nr++] = r0;
                if (r1 >= 0 && r1 <= 1 && r1 != r0) roots[nr++] = r1;
            }
        }
        for (int ri = 0; ri < nr; ri++) {
            Real tc = roots[ri];
            V3 pa = a0 + Pv * tc, pb = b0 + Qv * tc, e1 = pb - pa, n2 = cross(e1, D);
            Real n2l = dot(n2, n2);
            if (n2l < Real(1e-16)) continue;
            V3 wv = Sg - pa;
            Real u = dot(cross(wv, D), n2) / n2l, v = dot(cross(wv, e1), n2) / n2l;
            const Real EPS = Real(2e-2);
            if (u <= 0 || u > 1 || v < -EPS || v > Real(1) + EPS) continue;
            const V3 relV = (Pv + Qv) * Real(0.5f), nHit = cross(D, relV);
            const Real nLen = len(nHit);
            const V3 nEmit = nLen > Real(1e-8f) ? v3(nHit.x / nLen, nHit.y / nLen, nHit.z / nLen) : S.emitNcut;
            markAndEmit(g, a, b, (float)u, a1 + (b1 - a1) * u, nEmit);
            break;
        }
    }
    if (S.tearLen2 > 0) {
        for (size_t e = 0; e < S.gridEdges.size(); e++) {
            const GridEdge2& g = S.gridEdges[e];
            int a = cid(g.bx, g.by, g.bz), b = cid(g.bx + (g.axis == 0), g.by + (g.axis == 1), g.bz + (g.axis == 2));
            if (S.nbr[6 * a + 2 * g.axis + 1] < 0 || !S.active[a] || !S.active[b] || edgeIsCut(g)) continue;
            bool anyOcc = false;
            for (int s = 0; s < 4 && !anyOcc; s++) {
                int x = g.bx + ES_OFF[g.axis][s][0], y = g.by + ES_OFF[g.axis][s][1], z = g.bz + ES_OFF[g.axis][s][2];
                anyOcc = voxIn(x, y, z) && S.occupied[voxId(x, y, z)];
            }
            if (!anyOcc) continue;
            V3 d = S.pos[b] - S.pos[a];
            Real l2 = dot(d, d);
            V3 r = S.rest[b] - S.rest[a];
            Real tl2 = S.tearLen2 * (dot(r, r) / (Real(S.cd.voxelL) * Real(S.cd.voxelL)));
            // no grasp ring exists on this path: the release-decay state never arms
            if (S.edgeWasExempt[e]) { S.edgeWasExempt[e] = 0; S.edgeDecay[e] = 0; }
            if (l2 <= tl2) continue;
            S.tearMarks++;
            const Real l = std::sqrt(l2);
            markAndEmit(g, a, b, 0.5f, S.pos[a] + d * Real(0.5f), v3(d.x / l, d.y / l, d.z / l));
        }
    }
    severLinks();
    S.prevCorner = S.pos;
    return 0;
}

// ---------------------------------------------------------------------------------------------
// step / readback
// ---------------------------------------------------------------------------------------------
API int LCS_Step(float dt) {
    if (!S.physReady) return -1;
    auto t0 = std::chrono::steady_clock::now();
    int rc = beginFrame(dt);
    if (rc) return rc;
    int N = S.numSubsteps > 0 ? S.numSubsteps : 20;
    for (int n = 0; n < N; n++) {
        rc = substep();
        if (rc) return rc;
        if (S.cutReady) {
            const unsigned before = S.cutPoints;   // cut_surface_revision (V/cut.cu:1259-1262)
            ribbonTick();
            if (S.cutPoints != before && n + 1 < N) computeParticleFrames();   // V/physics.cu:368-379
        }
    }
    computeParticleFrames();   // LCS_Step's closing frames (plugin_api.cpp:125-134)
    if (S.profile) S.stepMs.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    return 0;
}
// plugin_api.cpp:157-165: frames from the post-sever lattice; the surface rebuild is not restated
API int LCS_Finalize() {
    if (!S.physReady) return -1;
    computeParticleFrames();
    buildSurfaceO();
    return 0;
}
API int LCS_GetCornerPos(float* out) {
    if (!S.reconReady || !out) return -1;
    for (int i = 0; i < S.N; i++) { out[3 * i] = (float)S.pos[i].x; out[3 * i + 1] = (float)S.pos[i].y; out[3 * i + 2] = (float)S.pos[i].z; }
    return 0;
}
API int ORC_GetCornerPos64(double* out) {
    if (!S.reconReady || !out) return -1;
    for (int i = 0; i < S.N; i++) { out[3 * i] = (double)S.pos[i].x; out[3 * i + 1] = (double)S.pos[i].y; out[3 * i + 2] = (double)S.pos[i].z; }
    return 0;
}
API int ORC_SetCornerPos(const float* in) {     // replay mode: overwrite the live positions (cut topology tests)
    if (!S.reconReady || !in) return -1;
    for (int i = 0; i < S.N; i++) S.pos[i] = v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
    return 0;
}
// The library's state restore (same arguments and checks): the replay tests load one state into the
// oracle, the CUDA library and (read back from it) the reference build's successor.
API int GBT_SetState(const float* pos3N, const float* vel3N, const int* nbr6N, const void* bendPairs, const int* active,
                     const unsigned* cutMaskV, const float* edgeCutT6N, const float* rot9N, int setRevision, unsigned revision) {
    if (!S.physReady) return ERR_NOT_READY;
    if ((cutMaskV || edgeCutT6N || setRevision) && !S.cutReady) return ERR_BAD_ARG;
    const size_t N = (size_t)S.N;
    for (size_t k = 0; pos3N && k < 3 * N; k++) if (!std::isfinite(pos3N[k])) return ERR_BAD_ARG;
    for (size_t k = 0; vel3N && k < 3 * N; k++) if (!std::isfinite(vel3N[k])) return ERR_BAD_ARG;
    for (size_t k = 0; rot9N && k < 9 * N; k++) if (!std::isfinite(rot9N[k])) return ERR_BAD_ARG;
    for (size_t i = 0; active && i < N; i++) if (active[i] != 0 && active[i] != 1) return ERR_BAD_ARG;
    if (nbr6N) {
        const long long stride[3] = {1, S.dx + 1, (long long)(S.dx + 1) * (S.dy + 1)};
        const int extent[3] = {S.dx, S.dy, S.dz};
        for (size_t i = 0; i < N; i++) {
            const int c[3] = {(int)(i % (S.dx + 1)), (int)(i / (S.dx + 1) % (S.dy + 1)), (int)(i / stride[2])};
            for (int s = 0; s < 6; s++) {
                const int v = nbr6N[6 * i + s], a = s >> 1, to = c[a] + ((s & 1) ? 1 : -1);
                if (v != -1 && (to < 0 || to > extent[a] || v != (long long)i + ((s & 1) ? stride[a] : -stride[a]))) return ERR_BAD_ARG;
            }
        }
    }
    if (cutMaskV) for (size_t v = 0; v < S.cutMask.size(); v++) if (cutMaskV[v] >> 12) return ERR_BAD_ARG;
    if (bendPairs) {
        const BendPair* in = (const BendPair*)bendPairs;
        for (size_t q = 0; q < S.bends.size(); q++) {
            BendPair a = S.bends[q], b = in[q];
            a.alive = b.alive = 0;
            if (std::memcmp(&a, &b, sizeof(BendPair)) != 0 || (in[q].alive != 0 && in[q].alive != 1)) return ERR_BAD_ARG;
        }
        for (size_t q = 0; q < S.bends.size(); q++) S.bends[q].alive = in[q].alive;
    }
    if (pos3N) for (size_t i = 0; i < N; i++) S.pos[i] = S.prev[i] = v3(pos3N[3 * i], pos3N[3 * i + 1], pos3N[3 * i + 2]);
    if (pos3N && S.cutReady) S.prevCorner = S.pos;
    if (vel3N) for (size_t i = 0; i < N; i++) S.vel[i] = v3(vel3N[3 * i], vel3N[3 * i + 1], vel3N[3 * i + 2]);
    if (nbr6N) std::memcpy(S.nbr.data(), nbr6N, 6 * N * sizeof(int));
    if (active) std::memcpy(S.active.data(), active, N * sizeof(int));
    if (cutMaskV) std::memcpy(S.cutMask.data(), cutMaskV, S.cutMask.size() * sizeof(unsigned));
    if (edgeCutT6N) std::memcpy(S.edgeCutT.data(), edgeCutT6N, 6 * N * sizeof(float));
    if (rot9N) for (size_t k = 0; k < 9 * N; k++) S.particleRot[k] = rot9N[k];
    if (setRevision) S.revision = revision;
    S.livenessStale = true; S.livenessRevision = 0xffffffffu;
    return 0;
}
API int GBT_GetActive(int* out) {
    if (!S.physReady || !out) return -1;
    std::memcpy(out, S.active.data(), (size_t)S.N * sizeof(int));
    return 0;
}
API int LCS_GetVelocities(float* out) {
    if (!S.physReady || !out) return -1;
    for (int i = 0; i < S.N; i++) { out[3 * i] = (float)S.vel[i].x; out[3 * i + 1] = (float)S.vel[i].y; out[3 * i + 2] = (float)S.vel[i].z; }
    return 0;
}
API int LCS_GetNbrIdx(int* out) {
    if (!S.physReady || !out) return -1;
    std::memcpy(out, S.nbr.data(), S.nbr.size() * sizeof(int));
    return 0;
}
API int LCS_GetBendPairs(void* out) {
    if (!S.physReady || !out) return -1;
    std::memcpy(out, S.bends.data(), S.bends.size() * sizeof(BendPair));
    return 0;
}
API int LCS_GetTopologyRevision(unsigned* r) {
    if (!r) return -1;
    *r = S.cutReady ? S.revision : 0;
    return 0;
}
API int LCS_GetCutEdgeFractions(float* out) {
    if (!S.cutReady || !out) return -1;
    std::memcpy(out, S.edgeCutT.data(), S.edgeCutT.size() * sizeof(float));
    return 0;
}
API int LCS_GetVoxelCutMask(unsigned* out) {
    if (!S.cutReady || !out) return -1;
    std::memcpy(out, S.cutMask.data(), S.cutMask.size() * sizeof(unsigned));
    return 0;
}
API int LCS_GetCutDebug(unsigned* out18, float* alpha) {
    if (!S.cutReady || !out18) return -1;
    std::memset(out18, 0, 18 * sizeof(unsigned));
    out18[15] = S.tearMarks; out18[16] = S.cutPoints;
    if (alpha) *alpha = S.cd.cutFPInterp;
    return 0;
}
API void LCS_ProfileEnable(int enabled) { S.profile = enabled != 0; S.stepMs.clear(); }
API void LCS_ProfileSections(int enabled) { (void)enabled; }
API int LCS_ProfileSectionsRead(char* text, int capacity) {   // the oracle times whole steps only
    if (!text || capacity < 1) return 1;
    text[0] = 0;
    return 0;
}
API int LCS_ProfileRead(int steps, float* ms) {
    if (!ms || steps <= 0 || (int)S.stepMs.size() < steps) return -1;
    double total = 0;
    for (int s = 0; s < steps; s++) total += S.stepMs[s];
    ms[0] = (float)total; ms[1] = 0; ms[2] = 0;
    return 0;
}
API void LCS_Shutdown() { resetCut(); resetPhysics(); S.reconReady = false; }
API double ORC_LogPositive(double x) { return (double)logPositive((Real)x); }   // the guarded bulk strain's log
API double ORC_PowMinusTwoThirds(double x) { return (double)powMinusTwoThirds((Real)x); }
API double ORC_AcosBend(double x) { return (double)acosBend((Real)x); }
API int ORC_GuardStats(long long* out3) {   // feasibility chain activity since the guard was armed
    if (!out3) return ERR_BAD_ARG;
    for (int k = 0; k < 3; k++) out3[k] = S.guardStats[k];
    return 0;
}
API int ORC_SetThreads(int n) {   // host threads of the colour sweeps (several oracle processes on one host)
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
    return n > 0 ? 0 : ERR_BAD_ARG;
}
API int ORC_Threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// cut topology of the live mesh: vertex duplication and re-colouring (a feature of this library)
#include "cut_topology_oracle.inc"

// differentiable rollout and its adjoint
#include "diff_oracle.inc"
