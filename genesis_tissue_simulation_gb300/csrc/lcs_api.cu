// LCS_* C ABI of the GB300 tissue solver: the drop-in for the reference plugin
// (endoscopic_tissue/native/vendor/src/plugin_api.cpp) on the plain XPBD path.
//
// One process-global session, as in the reference (endoscopic_tissue/native_backend.py:213-218).
// Host code builds the solver topology once (edge/bend/tet greedy colourings in the reference's
// emission order, Kuhn tets, rest shapes) and uploads it in colour order; LCS_Step then runs one
// persistent frame kernel per call.  Status codes follow the reference bands: 0 ok, -(cudaError),
// -1000..-1005 solver (xpbd_solver.h:25-33), -2000..-2004 physics (V/physics.cu:219-228), -3000..
// cut (V/cut.cu:1109-1427); -4001 marks entry points of the unified solver that this library does
// not provide, -4002 a device barrier that timed out.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>

#include "frame_kernels.h"
#include "mesh_build.h"
#include "session_view.h"
#include "surface.h"
#include "../../include/gbtissue.h"

using namespace gbt;

namespace {

// ---------------------------------------------------------------------------------------------
// session
// ---------------------------------------------------------------------------------------------
template <class T> struct DBuf {
    T* p = nullptr; size_t n = 0;
    cudaError_t alloc(size_t count) {
        release();
        n = count;
        return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    }
    cudaError_t upload(const T* h, size_t count, cudaStream_t s) {
        cudaError_t e = alloc(count);
        if (e == cudaSuccess && count) e = cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

struct Session {
    cudaStream_t stream = nullptr;
    int device = 0, smCount = 0, gridBlocks = 0, gridBlocksExt = 0;   // cooperative CTAs: plain / extended frame kernel
    bool reconReady = false, physReady = false, cutReady = false;
    int N = 0, dx = 0, dy = 0, dz = 0;
    std::vector<float> hostRest;            // rest lattice (3N), the first corner positions uploaded
    std::vector<float> skinT;               // [6N] skin crossing fraction per directed slot
    // physics parameters
    PhysicsInitDesc pd{};
    int numSubsteps = 20;
    float ks = 0, kb = 0, alpha = 0, betaS = 0, betaB = 0, youngE = 0, poisson = 0.45f, strainDamping = 0, omega = 1, damping = 0;
    float bulkDampingSeconds = 0.003125f, tissueHardening = 80.f;
    int volumePasses = 0; float minVolume = 0.f;
    // tissue guard buffers (LCS_SetTissueGuard): fibre multipliers, feasibility candidates and marks,
    // incident colour slots per node (CSR), two flags
    DBuf<float> fiberLambda; DBuf<float4> feasTarget; DBuf<int> needed, incOff, incTet; DBuf<unsigned> guardFlags;
    float lastH = -1.f;
    // topology sizes (host copies for diagnostics)
    int E = 0, B = 0, T = 0;
    std::vector<int> edgeColorOff, bendColorOff, tetColorOff;   // host copies [colors+1]
    std::vector<int> tetColorOrder;                             // colour slot -> storage index
    std::vector<int> tetIdsStorage;                             // [4T] storage order
    std::vector<float2> tetStiffStorage;                        // [T] (mu V, kappa V) storage order
    std::vector<int> edgeOwnerColor;                            // [E] owner slot per colour slot
    float typeB[6][9];
    // device buffers
    DBuf<float4> pos, prev, vel, ext, rest;
    DBuf<int> pinned, active, nbr, edgeColorOffD, bendColorOffD, tetColorOffD;
    DBuf<int2> edgeEnds; DBuf<float> edgeRest; DBuf<int> edgeOwner, edgeLive;
    DBuf<int4> bendIJK; DBuf<int> bendSrc, bendLive; DBuf<BendRecord> bendPairs;
    DBuf<int4> tetIds; DBuf<int> tetMeta, tetOwner, edgeSupport; DBuf<float2> tetAlpha, tetStiff;
    DBuf<unsigned> state;                   // [0] revision the liveness was derived at, [1] barrier counter, [2] status,
                                            // [3] current particle-frame buffer after the frame
    DBuf<float> rotA, rotB; int rotParity = 0;   // particle frames, 9 floats per node; rotParity: current buffer
    // dual-contouring surface (LCS_Init's voxel tables); rebuilt at LCS_Init and in LCS_Finalize
    bool surfaceReady = false, haveRestSurface = false;
    int nVox = 0, nSurfVox = 0, nSurfEdges = 0, triCapacity = 0, qefIters = 8, surfBlocks = 0;
    DBuf<int> voxelCorner, isectOff, isectCnt, surfVox, tri, nrmFixed, blockTotal;
    DBuf<IsectRec> isect; DBuf<int4> surfEdges; DBuf<float4> fp, fpRest, outAux; DBuf<float> outPos, outNrm;
    DBuf<unsigned> surfSync, triCount;
    DBuf<float4> cutFP; DBuf<int> cutNrmFixed, rawTri, wallCount; DBuf<int4> faces; int faceCap = 0;   // cut voxels' surface
    unsigned* hostState = nullptr;          // pinned mirror of state + cut counters
    DBuf<float> packedXyz;                  // node getters: xyz packed on the device (3N floats)
    // tool / contact
    bool toolArmed = false; ToolPose tool{}, toolFrom{};
    ContactParams cp{0.02f, 1.0e-7f, 0.5f, 0.045f, 0.25f};
    GraspParamsAbi gp{0.5f, 0.3f, 0.02f, 0.55f, 0.3f, 1.0e-7f, 0.02f, 0.5f, 0.045f, 0.25f, 0.25f, 1.0e-7f, 150.f, 0.045f, 1};
    int contactModel = 0;
    float muStatic = 0.f, muDynamic = 0.f, jawThickness = 0.f, contactRadius = 0.f;   // contact model 1
    // cut
    CutInitDesc cd{};
    DBuf<int4> gridEdges; DBuf<unsigned> occupied, cutMask, counters; DBuf<int> inside; DBuf<float> skinTD, edgeCutT;
    DBuf<int> conn;                         // [4096 x 9] components of the voxel corners per 12-bit cut mask
    DBuf<float4> cutRec;                    // [2 x 6N] cut points per directed lattice slot
    DBuf<int> brickList; DBuf<unsigned> brickCount; int nBricks = 0;   // ribbon-tick brick pre-cull
    bool bendsFollowLinks = false;          // every live bend pair (i; j, k) has the links i-j and i-k
    float emitNcut[3] = {0.f, 1.f, 0.f};    // last valid world cut normal of the blade
    bool toolSet = false, havePrev = false, pressure = false; CutToolDesc cutTool{};
    float tearLen2 = 0.f;
    // launch choice and profiling
    int launchMode = 0;                     // 0 automatic, 1 whole-GPU grid, 2 single CTA, 3 one cluster
    // automatic mode on a mesh that fits one CTA or one cluster: after the session's first frame,
    // one frame in each candidate shape (one CTA, whole GPU, one cluster) is timed and the fastest
    // kept (all give the same results bit for bit).  autoShape: -1 undecided, else kShape*.
    int autoShape = -1, autoTrial = 0; float autoMs[3] = {-1.f, -1.f, -1.f}; cudaEvent_t autoEv[2] = {nullptr, nullptr};
    int clockKHz = 2000000;                 // SM clock, for the barrier spin budget
    int maxStageBytes = 0;                  // shared memory one CTA may stage the node state in
    int maxClusterBytes = 0;                // dynamic shared memory of a session-cluster CTA
    int syncTestExtra = 0; float syncBudgetSeconds = 2.f;
    int lastFrameBlocks = 0;                // CTAs of the last frame if it ran on the whole-GPU grid, else 0
    DBuf<unsigned> floorSync;               // barrier-floor measurement: counter, status
    DBuf<int> uncovered0; bool fuseEdge0 = false;   // nodes ending no colour-0 edge; colour 0 is a matching
    bool profile = false; std::vector<cudaEvent_t> events; int profiledSteps = 0;
    // section profiler (xpbd_profile_sections, xpbd_solver.cu:30-60): device time per phase kind
    bool sections = false; DBuf<unsigned long long> phaseClock; std::vector<unsigned long long> phaseHost;
    double sectionMs[8] = {}; long long sectionCount[8] = {};
    // changes whenever the liveness flags must be derived again from scratch (a new mesh, a restored
    // state); LCS_StepNoAlloc keeps its liveness record only for the generation that wrote it
    unsigned long long generation = 0;
    DBuf<unsigned> bounds;                  // debug builds: out-of-range gather record (violations, index, site)
};
Session S;
unsigned long long g_sessionGeneration = 0;
}  // namespace
void forgetStepScratch();   // LCS_StepNoAlloc's cached scratch address (below)
namespace {

int cudaStatus(cudaError_t e) { return e == cudaSuccess ? 0 : -(int)e; }
#define CK(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) return -(int)_e; } while (0)

void freeCut() {
    S.gridEdges.release(); S.occupied.release(); S.cutMask.release(); S.counters.release(); S.inside.release();
    S.conn.release(); S.cutRec.release(); S.brickList.release(); S.brickCount.release(); S.nBricks = 0;
    S.cutFP.release(); S.cutNrmFixed.release(); S.rawTri.release(); S.wallCount.release(); S.faces.release(); S.faceCap = 0;
    S.emitNcut[0] = 0.f; S.emitNcut[1] = 1.f; S.emitNcut[2] = 0.f;
    S.skinTD.release(); S.edgeCutT.release();
    S.cutReady = false; S.toolSet = false; S.havePrev = false;
}
void freePhysics() {
    freeCut();
    releaseCutTopology();
    for (auto* b : {&S.prev, &S.vel, &S.ext}) b->release();
    for (auto* b : {&S.pinned, &S.active, &S.nbr, &S.edgeColorOffD, &S.bendColorOffD, &S.tetColorOffD, &S.edgeOwner, &S.edgeLive,
                    &S.bendSrc, &S.bendLive, &S.tetMeta, &S.tetOwner, &S.edgeSupport}) b->release();
    S.edgeEnds.release(); S.edgeRest.release(); S.bendIJK.release(); S.bendPairs.release(); S.tetIds.release();
    S.tetAlpha.release(); S.tetStiff.release(); S.state.release(); S.bounds.release(); S.floorSync.release();
    S.uncovered0.release(); S.fuseEdge0 = false;
    S.lastFrameBlocks = 0;
    S.fiberLambda.release(); S.feasTarget.release(); S.needed.release(); S.incOff.release(); S.incTet.release(); S.guardFlags.release();
    S.rotA.release(); S.rotB.release(); S.rotParity = 0;
    S.volumePasses = 0; S.minVolume = 0.f;
    // a live physics session's shutdown restores the tissue material defaults (physics.cu:218 ->
    // xpbd_shutdown, xpbd_solver.cu:3829); a material set before the first LCS_InitPhysics stays
    if (S.physReady) { S.tissueHardening = 80.f; S.bulkDampingSeconds = 0.003125f; }
    S.autoShape = -1; S.autoTrial = 0; S.autoMs[0] = S.autoMs[1] = S.autoMs[2] = -1.f;
    S.physReady = false; S.toolArmed = false; S.E = S.B = S.T = 0; S.lastH = -1.f;
}
void freeAll() {
    freePhysics();
    S.pos.release(); S.rest.release(); S.packedXyz.release();
    for (auto* b : {&S.voxelCorner, &S.isectOff, &S.isectCnt, &S.surfVox, &S.tri, &S.nrmFixed, &S.blockTotal}) b->release();
    S.isect.release(); S.surfEdges.release(); S.fp.release(); S.fpRest.release(); S.outAux.release();
    S.outPos.release(); S.outNrm.release(); S.surfSync.release(); S.triCount.release();
    S.surfaceReady = S.haveRestSurface = false;
    S.reconReady = false;
}

int ensureStream() {
    if (S.stream) return 0;
    CK(cudaGetDevice(&S.device));
    CK(cudaDeviceGetAttribute(&S.smCount, cudaDevAttrMultiProcessorCount, S.device));
    CK(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    CK(cudaMallocHost(&S.hostState, 8 * sizeof(unsigned)));
    int perSm = 0, perSmExt = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, frameKernelGrid, kFrameThreads, 0));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSmExt, frameKernelGridExt, kFrameThreads, 0));
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, S.device));
    S.maxStageBytes = optin;
    CK(cudaFuncSetAttribute((const void*)frameKernelBlock, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    CK(cudaFuncSetAttribute((const void*)frameKernelBlockExt, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    cudaFuncAttributes ca{};
    CK(cudaFuncGetAttributes(&ca, (const void*)frameKernelSessionCluster));
    S.maxClusterBytes = optin - (int)ca.sharedSizeBytes;   // dynamic bytes left beside its static shared memory
    CK(cudaFuncSetAttribute((const void*)frameKernelSessionCluster, cudaFuncAttributeMaxDynamicSharedMemorySize, S.maxClusterBytes));
    int khz = 0;
    if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, S.device) == cudaSuccess && khz > 0) S.clockKHz = khz;
    S.gridBlocks = std::max(1, perSm) * S.smCount;
    S.gridBlocksExt = std::max(1, perSmExt) * S.smCount;
    // one CTA per SM: the surface work is small, and every grid barrier costs in proportion to the CTAs
    int perSmSurface = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSmSurface, surfaceKernel, kSurfaceThreads, 0));
    if (perSmSurface < 1) return -(int)cudaErrorLaunchOutOfResources;
    S.surfBlocks = S.smCount;
    return 0;
}

// One rebuild of the dual-contouring surface from the live lattice (recon_build_static,
// V/dc_recon.cu:507-541).  With the cut buffers present, severed crossings are rebuilt from the
// current particle frames and cut voxels keep their QEF point.
int buildSurface() {
    if (!S.surfaceReady) return 0;
    SurfaceMesh m{};
    m.dx = S.dx; m.dy = S.dy; m.dz = S.dz;
    m.nSurfVox = S.nSurfVox; m.nEdges = S.nSurfEdges; m.triCapacity = S.triCapacity; m.qefIters = S.qefIters;
    m.haveRest = S.haveRestSurface ? 1 : 0;
    m.cutActive = S.cutReady ? 1 : 0;
    m.surfVox = S.surfVox.p; m.voxelCorner = S.voxelCorner.p; m.isectOff = S.isectOff.p; m.isectCnt = S.isectCnt.p;
    m.isect = S.isect.p; m.edges = S.surfEdges.p; m.pos = S.pos.p; m.rest = S.rest.p;
    m.nVox = S.nVox;
    if (S.cutReady) {
        m.nbr = S.nbr.p; m.rot = S.rotParity ? S.rotB.p : S.rotA.p; m.cutT = S.edgeCutT.p; m.cutMask = S.cutMask.p;
        m.conn = S.conn.p; m.occupied = S.occupied.p; m.inside = S.inside.p; m.skinT = S.skinTD.p; m.active = S.active.p;
        m.cutRec = S.cutRec.p; m.cutFP = S.cutFP.p; m.cutNrmFixed = S.cutNrmFixed.p; m.raw = S.rawTri.p;
        m.faces = S.faces.p; m.faceCap = S.faceCap; m.wallCount = S.wallCount.p;
    }
    m.fp = S.fp.p; m.fpRest = S.fpRest.p; m.nrmFixed = S.nrmFixed.p;
    m.tri = S.tri.p; m.triCount = S.triCount.p; m.blockTotal = S.blockTotal.p;
    m.outPos = S.outPos.p; m.outNrm = S.outNrm.p; m.outAux = S.outAux.p;
    unsigned* sync = S.surfSync.p;
    long long budget = (long long)((double)S.syncBudgetSeconds * 1e3 * S.clockKHz);
    CK(cudaMemsetAsync(sync, 0, 2 * sizeof(unsigned), S.stream));
    void* args[] = {&m, &sync, &budget};
    CK(cudaLaunchCooperativeKernel((const void*)surfaceKernel, dim3(S.surfBlocks), dim3(kSurfaceThreads), args, 0, S.stream));
    CK(cudaMemcpyAsync(S.hostState + 7, sync + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    return S.hostState[7] != 0u ? LCS_ERR_DEVICE_TIMEOUT : 0;
}

// Voxel tables of LCS_Init, checked so that every index the surface kernel follows stays inside
// its array; returns 0 or -1001.
int uploadSurface(const ReconInitDescAbi* d, const int* voxelCorner, const int* isectOffset, const int* isectCount,
                  const IsectAbi* isect, const int* surfaceEdges) {
    const int V = d->voxelCount, I = d->isectCount, E = d->surfaceEdgeCount, N = S.N;
    const int nx = S.dx + 1, nxy = (S.dx + 1) * (S.dy + 1);
    if (V != S.dx * S.dy * S.dz || I < 0 || E < 0 || d->qefIters < 0 || d->qefIters > 1000) return -1001;
    if (!voxelCorner || !isectOffset || !isectCount || (I > 0 && !isect) || (E > 0 && !surfaceEdges)) return -1001;
    for (size_t k = 0; k < (size_t)8 * V; k++) if (voxelCorner[k] < 0 || voxelCorner[k] >= N) return -1001;
    std::vector<int> surf;
    for (int v = 0; v < V; v++) {
        const int o = isectOffset[v], c = isectCount[v];
        if (c < 0 || c > 12 || o < 0 || (long long)o + c > I) return -1001;
        if (c > 0) surf.push_back(v);
    }
    for (int i = 0; i < I; i++) {
        const int a = isect[i].a, b = isect[i].b, dd = std::abs(b - a);
        if (a < 0 || a >= N || b < 0 || b >= N || !(dd == 1 || dd == nx || dd == nxy)) return -1001;
    }
    std::vector<int4> edges(E);
    for (int e = 0; e < E; e++) {
        const int* r = surfaceEdges + 8 * (size_t)e;
        const int axis = r[0], x = r[1], y = r[2], z = r[3], inA = r[4];
        const bool okx = axis == 0 ? (x >= 0 && x < S.dx) : (x >= 1 && x < S.dx);
        const bool oky = axis == 1 ? (y >= 0 && y < S.dy) : (y >= 1 && y < S.dy);
        const bool okz = axis == 2 ? (z >= 0 && z < S.dz) : (z >= 1 && z < S.dz);
        if (axis < 0 || axis > 2 || !okx || !oky || !okz || (inA != 0 && inA != 1)) return -1001;
        edges[e] = make_int4(axis | (inA << 2), x, y, z);
    }
    S.nVox = V; S.nSurfVox = (int)surf.size(); S.nSurfEdges = E; S.triCapacity = d->triCapacity; S.qefIters = d->qefIters;
    CK(S.voxelCorner.upload(voxelCorner, (size_t)8 * V, S.stream));
    CK(S.isectOff.upload(isectOffset, V, S.stream));
    CK(S.isectCnt.upload(isectCount, V, S.stream));
    CK(S.surfVox.upload(surf.data(), surf.size(), S.stream));
    CK(S.isect.upload((const IsectRec*)isect, I, S.stream));
    CK(S.surfEdges.upload(edges.data(), E, S.stream));
    const size_t idx = (size_t)3 * S.triCapacity;
    CK(S.fp.alloc(V)); CK(S.fpRest.alloc(V)); CK(S.nrmFixed.alloc((size_t)3 * V));
    CK(cudaMemsetAsync(S.fp.p, 0, (size_t)V * sizeof(float4), S.stream));
    CK(cudaMemsetAsync(S.fpRest.p, 0, (size_t)V * sizeof(float4), S.stream));
    CK(S.tri.alloc(idx)); CK(S.outPos.alloc(3 * idx)); CK(S.outNrm.alloc(3 * idx)); CK(S.outAux.alloc(idx));
    CK(S.blockTotal.alloc((size_t)2 * S.surfBlocks)); CK(S.surfSync.alloc(2)); CK(S.triCount.alloc(1));
    CK(cudaMemsetAsync(S.triCount.p, 0, sizeof(unsigned), S.stream));
    return 0;
}

int directedSlot(int a, int b) {
    int d = b - a, ad = d < 0 ? -d : d;
    int axis = ad == 1 ? 0 : (ad == S.dx + 1 ? 1 : 2);
    return 6 * a + 2 * axis + (d > 0 ? 1 : 0);
}

// Colour offsets [c0, c1, ..., cn] as the (begin, end) pair of every colour, the kernels' range form.
std::vector<int> colourRanges(const std::vector<int>& offsets) {
    std::vector<int> out;
    for (size_t c = 0; c + 1 < offsets.size(); c++) { out.push_back(offsets[c]); out.push_back(offsets[c + 1]); }
    return out;
}

int uploadFrameState() {
    std::vector<unsigned> st = {~0u, 0u, 0u, 0u};
    CK(S.state.upload(st.data(), 4, S.stream));
    return 0;
}

DeviceMesh deviceMesh() {
    DeviceMesh m{};
    m.nNodes = S.N; m.nodeBase = 0; m.dx = S.dx; m.dy = S.dy; m.dz = S.dz;
    m.pos = S.pos.p; m.prev = S.prev.p; m.vel = S.vel.p; m.ext = S.ext.p;
    m.pinned = S.pinned.p; m.active = S.active.p; m.nbr = S.nbr.p;
    m.nEdgeColors = (int)S.edgeColorOff.size() - 1; m.edgeRange = (const int2*)S.edgeColorOffD.p;
    m.edgeEnds = S.edgeEnds.p; m.edgeRest = S.edgeRest.p; m.edgeOwner = S.edgeOwner.p; m.edgeLive = S.edgeLive.p;
    m.uncovered0 = S.uncovered0.p; m.nUncovered0 = (int)S.uncovered0.n; m.fuseEdge0 = S.fuseEdge0 ? 1 : 0;
    m.nBendColors = (int)S.bendColorOff.size() - 1; m.bendRange = (const int2*)S.bendColorOffD.p;
    m.bendIJK = S.bendIJK.p; m.bendSrc = S.bendSrc.p; m.bendLive = S.bendLive.p; m.bendPairs = S.bendPairs.p;
    m.nBendPairs = (int)S.bendPairs.n;
    m.nTetColors = (int)S.tetColorOff.size() - 1; m.tetRange = (const int2*)S.tetColorOffD.p;
    m.tetIds = S.tetIds.p; m.tetMeta = S.tetMeta.p; m.tetOwner = S.tetOwner.p; m.tetAlpha = S.tetAlpha.p; m.tetStiff = S.tetStiff.p;
    m.edgeSupport = S.edgeSupport.p;
    std::memcpy(m.typeB, S.typeB, sizeof(S.typeB));
    m.fiberLambda = S.fiberLambda.p; m.feasTarget = S.feasTarget.p; m.needed = S.needed.p;
    m.incOff = S.incOff.p; m.incTet = S.incTet.p; m.guardFlags = S.guardFlags.p;
    m.particleRot[0] = S.rotA.p; m.particleRot[1] = S.rotB.p;
    m.bounds = S.bounds.p;
    return m;
}

CutParams cutParams() {
    CutParams c{};
    if (!S.cutReady) return c;
    c.nGridEdges = (int)S.gridEdges.n; c.gridEdges = S.gridEdges.p; c.occupied = S.occupied.p; c.cutMask = S.cutMask.p;
    c.inside = S.inside.p; c.skinT = S.skinTD.p; c.edgeCutT = S.edgeCutT.p; c.rest = S.rest.p; c.counters = S.counters.p;
    c.sx = S.cutTool.t2v2[0]; c.sy = S.cutTool.t2v2[1]; c.sz = S.cutTool.t2v2[2];
    c.ex = S.cutTool.t1v2[0]; c.ey = S.cutTool.t1v2[1]; c.ez = S.cutTool.t1v2[2];
    c.voxelL = S.cd.voxelL; c.tearLen2 = S.tearLen2; c.havePrev = S.havePrev ? 1 : 0;
    c.cutRec = S.cutRec.p; c.toolD = S.cutTool.d; c.ncx = S.emitNcut[0]; c.ncy = S.emitNcut[1]; c.ncz = S.emitNcut[2];
    c.brickList = S.brickList.p; c.brickCount = S.brickCount.p; c.nBricks = S.nBricks;
    c.skipSevered = S.bendsFollowLinks ? 1 : 0;
    return c;
}

// The frame kernel; when it runs on one CTA, the closing frame pass follows as a whole-GPU launch
// (*followUp set), so the host flips the parity the kernel leaves in state[3].
// Launch shapes of a frame: one CTA, the whole GPU, one thread-block cluster.
constexpr int kShapeBlock = 0, kShapeGrid = 1, kShapeCluster = 2;
constexpr int kSessionLogK = 3;   // 8 CTAs, the portable cluster size
size_t clusterBytes() {
    const size_t perCluster = (size_t)kSessionClusterThreads << kSessionLogK;
    return (((size_t)S.N + perCluster - 1) / perCluster) * kSessionClusterThreads * sizeof(float4);
}

// Which shapes can run this frame: one CTA only when the node state can be staged in its shared
// memory, the cluster only on plain frames whose positions fit its distributed shared memory.
struct Shapes { bool stage, clusterFits, usable[3]; size_t stageBytes; };
Shapes usableShapes(const FrameCoeffs& fc) {
    Shapes u{};
    u.stageBytes = (size_t)S.N * 2 * sizeof(float4);
    u.stage = u.stageBytes <= (size_t)S.maxStageBytes;
    u.clusterFits = clusterBytes() <= (size_t)S.maxClusterBytes;
    const bool plain = !fc.guarded && !fc.friction && !fc.cut;   // what the cluster shape runs
    u.usable[kShapeBlock] = u.stage; u.usable[kShapeGrid] = true; u.usable[kShapeCluster] = u.clusterFits && plain;
    return u;
}
// The shape the launch mode asks for; in automatic mode the kept trial winner, else (before the
// trials have decided) one CTA where the nodes stage, the whole GPU otherwise.
int requestedShape(const Shapes& u) {
    if (S.launchMode == 2) return kShapeBlock;
    if (S.launchMode == 3) return u.usable[kShapeCluster] ? kShapeCluster : kShapeGrid;
    if (S.launchMode == 1 || !(u.stage || u.clusterFits)) return kShapeGrid;
    if (S.autoShape >= 0) {
        if (u.usable[S.autoShape]) return S.autoShape;
        // e.g. a cluster choice on a frame with a blade: the faster usable other
        if (u.usable[kShapeBlock] && S.autoMs[kShapeBlock] >= 0.f && S.autoMs[kShapeBlock] <= S.autoMs[kShapeGrid]) return kShapeBlock;
        return kShapeGrid;
    }
    return u.stage ? kShapeBlock : kShapeGrid;
}

// One frame in `shape` on the session's stream, with `state` as its state words (the counter and
// status at [1], [2] must be zero) and m.tetAlpha as its compliances.  When the frame ran on one CTA
// or one cluster, the closing particle-frame pass follows as a whole-GPU launch (*followUp set), so
// the host flips the parity the kernel leaves in state[3].
int launchShape(int shape, const Shapes& u, const FrameCoeffs& fc, const DeviceMesh& m, unsigned* state, bool* followUp) {
    *followUp = false;
    CutParams cu = cutParams();
    ToolPose from = S.toolFrom, to = S.tool;
    ContactParams cp = S.cp;
    const bool ext = fc.guarded || fc.friction;
    if (shape == kShapeBlock) {
        FrameCoeffs f = fc;
        f.stageNodes = u.stage ? 1 : 0;
        f.closingPass = 0;
        (ext ? frameKernelBlockExt : frameKernelBlock)<<<1, kBlockThreads, u.stage ? u.stageBytes : 0, S.stream>>>(m, f, from, to, cp, cu, state);
        CK(cudaGetLastError());
    } else if (shape == kShapeCluster) {
        FrameCoeffs f = fc;
        f.closingPass = 0;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(1u << kSessionLogK); cfg.blockDim = dim3(kSessionClusterThreads); cfg.stream = S.stream;
        cfg.dynamicSmemBytes = clusterBytes();
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 1u << kSessionLogK; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr; cfg.numAttrs = 1;
        int logK = kSessionLogK;
        CK(cudaLaunchKernelEx(&cfg, frameKernelSessionCluster, m, f, from, to, cp, cu, state, logK));
    } else {
        DeviceMesh mm = m;
        FrameCoeffs f = fc;
        f.closingPass = 1;
        void* args[] = {&mm, (void*)&f, &from, &to, &cp, &cu, &state};
        CK(cudaLaunchCooperativeKernel(ext ? (const void*)frameKernelGridExt : (const void*)frameKernelGrid, dim3(ext ? S.gridBlocksExt : S.gridBlocks),
                                       dim3(kFrameThreads), args, 0, S.stream));
    }
    S.lastFrameBlocks = shape == kShapeGrid ? (ext ? S.gridBlocksExt : S.gridBlocks) : 0;
    if (shape != kShapeGrid && fc.rotations) {   // the closing particle-frame pass, on the whole GPU
        particleRotKernel<<<(S.N + 255) / 256, 256, 0, S.stream>>>(m, state + 3, 0);
        CK(cudaGetLastError());
        *followUp = true;
    }
    return 0;
}

// Coefficients of one frame of N substeps of length h (xpbd_begin_frame, xpbd_solver.cu:2481-2514,
// plus the switches of the substep's phases).
FrameCoeffs frameCoeffs(float h, int N) {
    FrameCoeffs fc{};
    fc.numSubsteps = N; fc.substeps = N; fc.firstSubstep = 0;
    float at = S.ks > 0.f ? 1.f / (S.ks * h * h) : 0.f;
    fc.velScale = (1.f - S.damping) / (1.f + S.alpha * h);
    fc.betaGammaHS = at * S.betaS * h;
    fc.alphaTilde = at;
    fc.doBend = (S.B > 0 && S.kb > 0.f) ? 1 : 0;
    fc.alphaB = fc.doBend ? 1.f / (S.kb * h * h) : 0.f;
    fc.betaGammaHB = fc.alphaB * S.betaB * h;
    fc.h = h; fc.invH = 1.f / h; fc.invH2 = 1.f / (h * h);
    fc.doStrain = (S.T > 0 && S.youngE > 0.f) ? 1 : 0;
    fc.fallback = (fc.doStrain && S.ks <= 0.f) ? 1 : 0;
    fc.doEdges = (S.ks > 0.f || fc.fallback) ? 1 : 0;
    fc.fallbackInvEh2 = fc.fallback ? 1.f / (S.youngE * h * h) : 0.f;
    fc.perpDamp = S.betaS > 0.f ? 1 : 0;
    fc.betaS = S.betaS;
    fc.omega = S.omega;
    fc.dampingOverH = fmaxf(0.f, S.strainDamping) / h;
    fc.guarded = (S.volumePasses > 0 && S.T > 0) ? 1 : 0;
    fc.volumePasses = S.volumePasses;
    fc.tensileStrength = S.tissueHardening;
    fc.bulkDampingOverH = S.bulkDampingSeconds / h;
    fc.invScale = 1.f / (1.f + fc.dampingOverH); fc.invBulkScale = 1.f / (1.f + fc.bulkDampingOverH);
    fc.minVolume = S.minVolume;
    fc.contact = (S.toolArmed && S.contactModel == 0) ? 1 : 0;
    fc.friction = (S.toolArmed && S.contactModel == 1) ? 1 : 0;
    fc.muS = S.muStatic; fc.muD = S.muDynamic; fc.jawThickness = S.jawThickness; fc.contactRadius = S.contactRadius;
    fc.contactAlphaH2 = S.cp.contactAlpha / (h * h);
    fc.cut = (S.cutReady && S.toolSet && !S.pressure) ? 1 : 0;
    fc.spinBudget = (long long)((double)S.syncBudgetSeconds * 1e3 * S.clockKHz);
    fc.syncTestExtra = S.syncTestExtra;
    fc.rotations = 1; fc.rotParity = S.rotParity;
    return fc;
}

// LCS_Step's frame: the shape of the launch mode, and in automatic mode on a mesh that fits one
// CTA or one cluster, the session's 2nd to 4th frames each timed in one candidate shape.
int launchFrame(const FrameCoeffs& fc, bool* followUp) {
    unsigned* state = S.state.p;
    CK(cudaMemsetAsync(state + 1, 0, 2 * sizeof(unsigned), S.stream));
    if (S.brickCount.p) CK(cudaMemsetAsync(S.brickCount.p, 0, sizeof(unsigned), S.stream));
    const Shapes u = usableShapes(fc);
    int shape = requestedShape(u);
    int timed = -1;   // the automatic trial shape timed in this frame
    const bool trials = S.launchMode == 0 && (u.stage || u.clusterFits) && S.autoShape < 0;
    if (trials && S.autoTrial >= 1 && S.autoTrial <= 3) {
        timed = S.autoTrial - 1;   // 0 one CTA, 1 whole GPU, 2 cluster
        if (u.usable[timed]) shape = timed;
        else { timed = -1; shape = kShapeGrid; }
    } else if (trials && S.autoTrial > 3) {
        shape = kShapeGrid;
    }
    if (timed >= 0) {
        if (!S.autoEv[0]) { CK(cudaEventCreate(&S.autoEv[0])); CK(cudaEventCreate(&S.autoEv[1])); }
        CK(cudaEventRecord(S.autoEv[0], S.stream));
    }
    int rc = launchShape(shape, u, fc, deviceMesh(), state, followUp);
    if (rc) return rc;
    if (timed >= 0) CK(cudaEventRecord(S.autoEv[1], S.stream));
    if (trials) {   // record the trial
        S.autoTrial++;
        if (timed >= 0) {
            CK(cudaEventSynchronize(S.autoEv[1]));
            CK(cudaEventElapsedTime(&S.autoMs[timed], S.autoEv[0], S.autoEv[1]));
        }
        if (S.autoTrial > 3) {   // every candidate had its frame: keep the fastest measured
            int best = kShapeGrid;
            for (int k = 0; k < 3; k++)
                if (S.autoMs[k] >= 0.f && (S.autoMs[best] < 0.f || S.autoMs[k] < S.autoMs[best])) best = k;
            S.autoShape = best;
        }
    }
    return 0;
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
LCS_API int LCS_Init(const ReconInitDescAbi* desc, const float* cornerPos, const int* voxelCorner, const int* voxelIsectOffset,
                     const int* voxelIsectCount, const void* isect, const void* surfaceEdges) {
    freeAll();
    forgetStepScratch();
    if (!desc) return -1000;
    if (desc->voxelCount <= 0 || desc->cornerCount <= 0 || desc->triCapacity <= 0 || !cornerPos) return -1001;
    if ((long long)(desc->dimsX + 1) * (desc->dimsY + 1) * (desc->dimsZ + 1) != desc->cornerCount) return -1001;
    int rc = ensureStream();
    if (rc) return rc;
    S.N = desc->cornerCount; S.dx = desc->dimsX; S.dy = desc->dimsY; S.dz = desc->dimsZ;
    S.hostRest.assign(cornerPos, cornerPos + 3 * (size_t)S.N);
    std::vector<float4> p4(S.N);
    for (int i = 0; i < S.N; i++) p4[i] = make_float4(cornerPos[3 * i], cornerPos[3 * i + 1], cornerPos[3 * i + 2], 0.f);
    CK(S.pos.upload(p4.data(), S.N, S.stream));
    CK(S.rest.upload(p4.data(), S.N, S.stream));
    CK(S.packedXyz.alloc((size_t)3 * S.N));
    S.skinT.assign((size_t)6 * S.N, -1.f);
    const IsectAbi* is = (const IsectAbi*)isect;
    for (int i = 0; is && i < desc->isectCount; i++) {
        S.skinT[directedSlot(is[i].a, is[i].b)] = is[i].t;
        S.skinT[directedSlot(is[i].b, is[i].a)] = 1.f - is[i].t;
    }
    S.reconReady = true;
    if (voxelCorner) {   // the static surface of the rest lattice, then its rest snapshot (V/dc_recon.cu:612-621)
        rc = uploadSurface(desc, voxelCorner, voxelIsectOffset, voxelIsectCount, is, (const int*)surfaceEdges);
        if (rc) { freeAll(); return rc; }
        S.surfaceReady = true;
        rc = buildSurface();
        if (rc) { freeAll(); return rc; }
        CK(cudaMemcpyAsync(S.fpRest.p, S.fp.p, (size_t)S.nVox * sizeof(float4), cudaMemcpyDeviceToDevice, S.stream));
        S.haveRestSurface = true;
    }
    CK(cudaStreamSynchronize(S.stream));
    return 0;
}

LCS_API int LCS_PhysicsAbiVersion() { return (int)sizeof(PhysicsInitDesc); }
LCS_API int LCS_GraspToolAbiVersion() { return (int)sizeof(ToolPose); }
LCS_API int LCS_ContactModelVersion() { return 28; }

LCS_API int LCS_InitPhysics(const PhysicsInitDesc* desc, const float* mass, const int* pinned, const int* active, const float* extForce,
                            const int* nbrIdx, const float* restNbr, const void* bendPairs) {
    freePhysics();
    if (!desc) return -2000;
    if (!std::isfinite(desc->youngE) || desc->youngE < 0.f || !std::isfinite(desc->poisson) || desc->poisson < 0.f ||
        desc->poisson >= 0.5f || !std::isfinite(desc->strainDamping) || desc->strainDamping < 0.f) return -2004;
    const int cc = desc->cornerCount, bpc = desc->bendPairCount;
    if (cc <= 0) return -2001;
    if (!S.reconReady || cc != S.N) return -2002;
    if (!mass || !pinned || !active || !extForce || !nbrIdx || !restNbr || bpc < 0 || (bpc > 0 && !bendPairs)) return XPBD_ERR_BAD_ARG;
    S.pd = *desc;
    S.numSubsteps = desc->maxSubsteps > 0 ? desc->maxSubsteps : 20;
    S.omega = 1.f; S.damping = 0.f; S.ks = desc->ks; S.kb = desc->kb; S.alpha = desc->alpha; S.betaS = desc->cs; S.betaB = desc->cb;
    S.youngE = desc->youngE; S.poisson = desc->poisson; S.strainDamping = desc->strainDamping;

    MeshInput in{S.dx, S.dy, S.dz, S.hostRest.data(), mass, pinned, active, extForce, nbrIdx, restNbr, bendPairs, bpc,
                 S.youngE, S.poisson};
    HostMesh hm;
    int rc = buildHostMesh(in, hm);
    if (rc) return rc;
    const int E = hm.E, B = hm.B, T = hm.T;
    S.edgeColorOff = hm.edgeColorOff; S.bendColorOff = hm.bendColorOff; S.tetColorOff = hm.tetColorOff;
    S.edgeOwnerColor = hm.edgeOwner; S.tetColorOrder = hm.tetColorOrder;
    S.tetIdsStorage = hm.tetIdsStorage; S.tetStiffStorage = hm.tetStiffStorage;
    std::memcpy(S.typeB, hm.typeB, sizeof(S.typeB));
    S.E = E; S.B = B; S.T = T;
    const BendRecord* bp = (const BendRecord*)bendPairs;
    S.bendsFollowLinks = true;
    for (int q = 0; q < bpc && S.bendsFollowLinks; q++) {
        if (bp[q].alive == 0) continue;
        const int i = bp[q].i;
        bool hj = false, hk = false;
        if (i >= 0 && i < cc)
            for (int t = 0; t < 6; t++) { hj = hj || nbrIdx[6 * (size_t)i + t] == bp[q].j; hk = hk || nbrIdx[6 * (size_t)i + t] == bp[q].k; }
        S.bendsFollowLinks = hj && hk && bp[q].j >= 0 && bp[q].k >= 0;
    }
    std::vector<float4> zero4(cc, make_float4(0, 0, 0, 0));
    CK(S.pos.upload(hm.pos.data(), cc, S.stream));
    CK(S.prev.upload(hm.pos.data(), cc, S.stream));
    CK(S.vel.upload(zero4.data(), cc, S.stream));
    CK(S.ext.upload(hm.ext.data(), cc, S.stream));
    CK(S.pinned.upload(pinned, cc, S.stream));
    CK(S.active.upload(active, cc, S.stream));
    CK(S.nbr.upload(nbrIdx, (size_t)6 * cc, S.stream));
    std::vector<int> edgeRanges = colourRanges(S.edgeColorOff), bendRanges = colourRanges(S.bendColorOff),
                     tetRanges = colourRanges(S.tetColorOff);
    CK(S.edgeColorOffD.upload(edgeRanges.data(), edgeRanges.size(), S.stream));
    CK(S.edgeEnds.upload(hm.edgeEnds.data(), E, S.stream));
    {   // nodes that end no colour-0 edge; the fusion needs colour 0 to be a matching
        std::vector<unsigned char> ends(cc, 0);
        bool matching = S.edgeColorOff.size() > 1;
        for (int e = matching ? S.edgeColorOff[0] : 0; matching && e < S.edgeColorOff[1]; e++) {
            const int2 ij = hm.edgeEnds[e];
            if (ij.x < 0 || ij.y < 0 || ij.x >= (int)cc || ij.y >= (int)cc || ends[ij.x] || ends[ij.y]) matching = false;
            else ends[ij.x] = ends[ij.y] = 1;
        }
        std::vector<int> rest;
        for (int i = 0; matching && i < (int)cc; i++) if (!ends[i]) rest.push_back(i);
        CK(S.uncovered0.upload(rest.data(), rest.size(), S.stream));
        S.fuseEdge0 = matching;
    }
    CK(S.edgeRest.upload(hm.edgeRest.data(), E, S.stream));
    CK(S.edgeOwner.upload(hm.edgeOwner.data(), E, S.stream));
    std::vector<int> ones(std::max(std::max(E, B), 1), 1);
    CK(S.edgeLive.upload(ones.data(), E, S.stream));
    CK(S.bendColorOffD.upload(bendRanges.data(), bendRanges.size(), S.stream));
    CK(S.bendIJK.upload(hm.bendIJK.data(), B, S.stream));
    CK(S.bendSrc.upload(hm.bendSrc.data(), B, S.stream));
    CK(S.bendLive.upload(ones.data(), B, S.stream));
    CK(S.bendPairs.upload(bp, bpc, S.stream));
    CK(S.tetColorOffD.upload(tetRanges.data(), tetRanges.size(), S.stream));
    CK(S.tetIds.upload(hm.tetIds.data(), T, S.stream));
    CK(S.tetMeta.upload(hm.tetMeta.data(), T, S.stream));
    CK(S.tetOwner.upload(hm.tetOwner.data(), (size_t)3 * T, S.stream));
    CK(S.tetStiff.upload(hm.tetStiff.data(), T, S.stream));
    CK(S.tetAlpha.alloc(T));
    std::vector<int> zeros((size_t)6 * cc, 0);
    CK(S.edgeSupport.upload(zeros.data(), (size_t)6 * cc, S.stream));
    std::vector<float> identity((size_t)9 * cc, 0.f);   // particle frames start at the identity (V/physics.cu:258-267)
    for (int i = 0; i < cc; i++) identity[9 * (size_t)i] = identity[9 * (size_t)i + 4] = identity[9 * (size_t)i + 8] = 1.f;
    CK(S.rotA.upload(identity.data(), identity.size(), S.stream));
    CK(S.rotB.upload(identity.data(), identity.size(), S.stream));
    S.rotParity = 0;
    rc = uploadFrameState();
    if (rc) return rc;
#ifdef GBT_DEBUG_BOUNDS
    CK(S.bounds.alloc(3));
    CK(cudaMemsetAsync(S.bounds.p, 0, 3 * sizeof(unsigned), S.stream));
#endif
    CK(cudaStreamSynchronize(S.stream));
    S.generation = ++g_sessionGeneration;
    S.physReady = true;
    return 0;
}

LCS_API int LCS_SetGravity(float gx, float gy, float gz) {
    if (!S.physReady) return XPBD_ERR_NOT_READY;
    if (!std::isfinite(gx) || !std::isfinite(gy) || !std::isfinite(gz)) return XPBD_ERR_BAD_ARG;
    gravityKernel<<<(S.N + 255) / 256, 256, 0, S.stream>>>(S.N, gx, gy, gz, S.ext.p);
    return cudaStatus(cudaGetLastError());
}

LCS_API int LCS_SetTetStiffness(int count, const float* muV, const float* kappaV) {
    if (!S.physReady) return XPBD_ERR_NOT_READY;
    if (count != S.T || !muV || !kappaV) return XPBD_ERR_BAD_ARG;
    for (int t = 0; t < count; t++)
        if (!(muV[t] > 0.f) || !(kappaV[t] > 0.f) || !std::isfinite(muV[t]) || !std::isfinite(kappaV[t])) return XPBD_ERR_BAD_ARG;
    std::vector<float2> c(count);
    for (int k = 0; k < count; k++) {
        int t = S.tetColorOrder[k];
        c[k] = make_float2(muV[t], kappaV[t]);
        S.tetStiffStorage[t] = c[k];
    }
    CK(cudaMemcpyAsync(S.tetStiff.p, c.data(), count * sizeof(float2), cudaMemcpyHostToDevice, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    S.lastH = -1.f;
    return 0;
}

LCS_API int LCS_GetTetStiffness(float* muV, float* kappaV) {
    if (!S.physReady || !muV || !kappaV) return XPBD_ERR_BAD_ARG;
    for (int t = 0; t < S.T; t++) { muV[t] = S.tetStiffStorage[t].x; kappaV[t] = S.tetStiffStorage[t].y; }
    return 0;
}
LCS_API int LCS_TetCount() { return S.physReady ? S.T : 0; }
LCS_API int LCS_TetColorCount() { return S.physReady ? (int)S.tetColorOff.size() - 1 : 0; }
LCS_API int LCS_EdgeColorCount() { return S.physReady ? (int)S.edgeColorOff.size() - 1 : 0; }
LCS_API int LCS_EdgeCount() { return S.physReady ? S.E : 0; }
LCS_API int LCS_GetTetIds(int* out) {
    if (!S.physReady || !out) return XPBD_ERR_BAD_ARG;
    std::memcpy(out, S.tetIdsStorage.data(), S.tetIdsStorage.size() * sizeof(int));
    return 0;
}
LCS_API int LCS_GetTetColors(int* out) {
    if (!S.physReady || !out) return XPBD_ERR_BAD_ARG;
    for (size_t c = 0; c + 1 < S.tetColorOff.size(); c++)
        for (int k = S.tetColorOff[c]; k < S.tetColorOff[c + 1]; k++) out[S.tetColorOrder[k]] = (int)c;
    return 0;
}
LCS_API int LCS_GetEdgeColors(int* out6N) {
    if (!S.physReady || !out6N) return XPBD_ERR_BAD_ARG;
    std::fill(out6N, out6N + 6 * (size_t)S.N, -1);
    for (size_t c = 0; c + 1 < S.edgeColorOff.size(); c++)
        for (int k = S.edgeColorOff[c]; k < S.edgeColorOff[c + 1]; k++) out6N[S.edgeOwnerColor[k]] = (int)c;
    return 0;
}

LCS_API void LCS_SetGraspParams(const GraspParamsAbi* p) {
    if (!p) return;
    S.gp = *p;
    S.cp.jawGapClosed = p->jawGapClosed; S.cp.contactAlpha = p->contactAlpha; S.cp.ccdVelThresh = p->ccdVelThresh;
    S.cp.ccdMaxDisp = p->ccdMaxDisp; S.cp.ccdOmega = p->ccdOmega;
}
LCS_API int LCS_SetContactModel(int enabled, float muS, float muD, float thickness, float radius) {
    if (!S.physReady) return XPBD_ERR_NOT_READY;
    if (enabled < 0 || enabled > 2 || !std::isfinite(muS) || !std::isfinite(muD) || !std::isfinite(thickness) || !std::isfinite(radius) ||
        muS < 0 || muD < 0 || muD > muS || thickness <= 0 || radius < 0) return XPBD_ERR_BAD_ARG;
    if (enabled == 2) return LCS_ERR_UNSUPPORTED;   // anchor assist belongs to the unified grasp solver
    S.contactModel = enabled;
    S.muStatic = muS; S.muDynamic = muD; S.jawThickness = thickness; S.contactRadius = radius;
    return 0;
}
LCS_API int LCS_SetTissueGuard(float minimum, int passes, int count, const int* inside, int capture) {
    (void)capture;
    if (!S.physReady || S.lastH > 0 || !std::isfinite(minimum) || minimum < 0 || minimum > .95f || passes < 0 || passes > 4 ||
        count != S.N || !inside) return XPBD_ERR_BAD_ARG;
    // incident colour slots of every node (the feasibility line search reads each vertex's tets)
    std::vector<int> off(S.N + 1, 0), inc((size_t)4 * S.T);
    for (int k = 0; k < S.T; k++)
        for (int c = 0; c < 4; c++) off[S.tetIdsStorage[4 * (size_t)S.tetColorOrder[k] + c] + 1]++;
    for (int i = 0; i < S.N; i++) off[i + 1] += off[i];
    std::vector<int> cursor(off.begin(), off.end() - 1);
    for (int k = 0; k < S.T; k++)
        for (int c = 0; c < 4; c++) inc[cursor[S.tetIdsStorage[4 * (size_t)S.tetColorOrder[k] + c]]++] = k;
    CK(S.incOff.upload(off.data(), off.size(), S.stream));
    CK(S.incTet.upload(inc.data(), inc.size(), S.stream));
    CK(S.fiberLambda.alloc((size_t)6 * std::max(S.T, 1)));
    CK(S.feasTarget.alloc(S.N));
    CK(S.needed.alloc(S.N));
    CK(S.guardFlags.alloc(2));
    CK(cudaMemsetAsync(S.needed.p, 0, S.N * sizeof(int), S.stream));
    CK(cudaMemsetAsync(S.guardFlags.p, 0, 2 * sizeof(unsigned), S.stream));
    CK(cudaStreamSynchronize(S.stream));
    S.volumePasses = passes;
    S.minVolume = minimum;
    return 0;
}
LCS_API int LCS_SetTissueMaterial(float strength, float bulkDamping) {
    if (!S.physReady || S.lastH > 0 || !std::isfinite(strength) || strength < 0 || strength > 1000 || !std::isfinite(bulkDamping) ||
        bulkDamping < 0 || bulkDamping > 1) return XPBD_ERR_BAD_ARG;
    S.tissueHardening = strength; S.bulkDampingSeconds = bulkDamping;
    return 0;
}
LCS_API int LCS_SetGraspTool(const void* toolState) {
    if (!S.physReady || !toolState) return -1;
    ToolPose t;
    std::memcpy(&t, toolState, sizeof(t));
    S.toolFrom = S.toolArmed ? S.tool : t;
    S.tool = t;
    S.toolArmed = true;
    if (t.grasp01 > S.gp.graspThreshold) return LCS_ERR_UNSUPPORTED;   // a capture starts the grasp solver
    return 0;
}

// ---------------------------------------------------------------------------------------------
// cut
// ---------------------------------------------------------------------------------------------
LCS_API int LCS_InitCut(const CutInitDesc* desc, const void* conn4096, const void* gridEdges, const int* voxelOccupied,
                        const int* cornerInside) {
    freeCut();
    if (!desc) return -3000;
    if (desc->voxelCount <= 0 || desc->cornerCount <= 0) return -3001;
    if (!S.physReady || desc->cornerCount != S.N || desc->dimsX != S.dx || desc->dimsY != S.dy || desc->dimsZ != S.dz) return -3002;
    if (desc->voxelCount != S.dx * S.dy * S.dz || !voxelOccupied || !cornerInside || desc->gridEdgeCount < 0 ||
        (desc->gridEdgeCount > 0 && !gridEdges)) return -3001;
    S.cd = *desc;
    CK(S.gridEdges.upload((const int4*)gridEdges, desc->gridEdgeCount, S.stream));
    CK(S.occupied.upload((const unsigned*)voxelOccupied, desc->voxelCount, S.stream));
    CK(S.cutMask.alloc(desc->voxelCount));
    CK(cudaMemsetAsync(S.cutMask.p, 0, desc->voxelCount * sizeof(unsigned), S.stream));
    CK(S.inside.upload(cornerInside, S.N, S.stream));
    CK(S.skinTD.upload(S.skinT.data(), S.skinT.size(), S.stream));
    std::vector<float> minus((size_t)6 * S.N, -1.f);
    CK(S.edgeCutT.upload(minus.data(), minus.size(), S.stream));
    CK(S.counters.alloc(4));
    CK(cudaMemsetAsync(S.counters.p, 0, 4 * sizeof(unsigned), S.stream));
    // connectivity table (Conn4096Gpu, V/cut.cuh:50-56): component count and component of each local
    // corner for every cut mask; checked so every feature-point slot 8 v + component stays in range
    if (conn4096) {
        const int* t = (const int*)conn4096;
        for (int k = 0; k < 4096; k++) {
            const int n = t[9 * k];
            if (n < 0 || n > 8) return -3001;
            for (int c = 0; c < 8; c++) if (t[9 * k + 1 + c] < 0 || t[9 * k + 1 + c] >= 8) return -3001;
        }
        CK(S.conn.upload(t, (size_t)9 * 4096, S.stream));
    }
    CK(S.cutRec.alloc((size_t)12 * S.N));
    CK(cudaMemsetAsync(S.cutRec.p, 0, (size_t)12 * S.N * sizeof(float4), S.stream));
    {   // the ribbon tick may enumerate edges by lattice bricks only if the edge list is the full
        // interior set (every edge whose four incident voxels exist), each once
        const int d[3] = {S.dx, S.dy, S.dz};
        long long expected = 0;
        for (int a = 0; a < 3; a++) expected += (long long)d[a] * (d[(a + 1) % 3] - 1) * (d[(a + 2) % 3] - 1);
        bool full = expected == desc->gridEdgeCount;
        std::vector<unsigned char> seen(full ? (size_t)3 * S.N : 0, 0);
        const int* g = (const int*)gridEdges;
        for (int e = 0; full && e < desc->gridEdgeCount; e++) {
            const int axis = g[4 * e], c[3] = {g[4 * e + 1], g[4 * e + 2], g[4 * e + 3]};
            if (axis < 0 || axis > 2) { full = false; break; }
            for (int a = 0; a < 3; a++)
                if (a == axis ? (c[a] < 0 || c[a] >= d[a]) : (c[a] < 1 || c[a] >= d[a])) full = false;
            if (!full) break;
            const size_t slot = 3 * ((size_t)c[0] + (S.dx + 1) * ((size_t)c[1] + (S.dy + 1) * (size_t)c[2])) + axis;
            if (seen[slot]) full = false;
            seen[slot] = 1;
        }
        if (full) {
            const int k = 4;
            S.nBricks = ((S.dx + k - 1) / k) * ((S.dy + k - 1) / k) * ((S.dz + k - 1) / k);
            CK(S.brickList.alloc(S.nBricks)); CK(S.brickCount.alloc(1));
            CK(cudaMemsetAsync(S.brickCount.p, 0, sizeof(unsigned), S.stream));
        }
    }
    if (S.surfaceReady && S.conn.p) {   // the cut voxels' share of the surface: component points, walls
        CK(S.cutFP.alloc((size_t)8 * S.nVox)); CK(S.cutNrmFixed.alloc((size_t)24 * S.nVox)); CK(S.wallCount.alloc((size_t)S.nVox));
        CK(cudaMemsetAsync(S.cutFP.p, 0, (size_t)8 * S.nVox * sizeof(float4), S.stream));
        CK(S.rawTri.alloc((size_t)3 * S.triCapacity));
        int cap = 1;
        while (cap < 2 * S.triCapacity) cap <<= 1;
        CK(S.faces.alloc(cap));
        S.faceCap = cap;
    }
    float tau = desc->tearStretchRatio;
    S.tearLen2 = (tau >= 1.0f && tau == tau) ? (tau * desc->voxelL) * (tau * desc->voxelL) : 0.f;
    CK(cudaStreamSynchronize(S.stream));
    S.cutReady = true;
    S.generation = ++g_sessionGeneration;   // the revision counter restarts at 0 with the cut module
    return 0;
}
LCS_API void LCS_SetTool(const CutToolDesc* tool) {
    if (!tool) return;
    S.cutTool = *tool;
    if (tool->valid != 0) { S.emitNcut[0] = tool->ncut[0]; S.emitNcut[1] = tool->ncut[1]; S.emitNcut[2] = tool->ncut[2]; }
    if (!S.toolSet && S.cutReady) S.havePrev = true;   // the snapshot is the current positions
    S.toolSet = true;
}
LCS_API void LCS_SetPressureCutMode(int enabled) { S.pressure = enabled != 0; }

LCS_API int LCS_DetectCut() {
    if (!S.cutReady || !S.toolSet || S.pressure) return 0;
    int n = (int)S.gridEdges.n;
    if (n <= 0) return 0;
    DeviceMesh m = deviceMesh();
    CutParams cu = cutParams();
    QuadTool q{};
    const CutToolDesc& c = S.cutTool;
    auto v = [](const float* a) { f3 r; r.x = a[0]; r.y = a[1]; r.z = a[2]; return r; };
    q.t1[0] = v(c.t1v0); q.t1[1] = v(c.t1v1); q.t1[2] = v(c.t1v2);
    q.t2[0] = v(c.t2v0); q.t2[1] = v(c.t2v1); q.t2[2] = v(c.t2v2);
    q.lo = v(c.aabbMin); q.hi = v(c.aabbMax); q.ncut = v(c.ncut); q.valid = c.valid;
    detectQuadKernel<<<(n + 255) / 256, 256, 0, S.stream>>>(m, cu, q, S.rotParity ? S.rotB.p : S.rotA.p);
    severKernel<<<(n + 255) / 256, 256, 0, S.stream>>>(m, cu);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(S.stream));
    return 0;
}

// ---------------------------------------------------------------------------------------------
// step
// ---------------------------------------------------------------------------------------------
LCS_API int LCS_Step(float dt) {
    if (!S.physReady) return -1;
    const int N = S.numSubsteps > 0 ? S.numSubsteps : 1;
    float h = dt / (float)N;
    if (!(h > 0.f) || !std::isfinite(h)) return XPBD_ERR_BAD_DT;
    FrameCoeffs fc = frameCoeffs(h, N);
    if (fc.doStrain && h != S.lastH) {
        tetAlphaKernel<<<(S.T + 255) / 256, 256, 0, S.stream>>>(S.T, fc.invH2, S.tetStiff.p, S.tetAlpha.p);
        CK(cudaGetLastError());
        S.lastH = h;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (S.profile) {
        CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, S.stream));
    }
    size_t records = (size_t)N * kPhaseRecordsPerSubstep;
    if (S.sections) {
        if (S.phaseClock.n < records) CK(S.phaseClock.alloc(records));
        CK(cudaMemsetAsync(S.phaseClock.p, 0, records * sizeof(unsigned long long), S.stream));
        fc.phaseClock = S.phaseClock.p;
    }
    bool followUp = false;
    int rc = launchFrame(fc, &followUp);
    if (rc) return rc;
    if (S.profile) { CK(cudaEventRecord(e1, S.stream)); S.events.push_back(e0); S.events.push_back(e1); }
    CK(cudaMemcpyAsync(S.hostState, S.state.p, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    if (S.sections) {
        S.phaseHost.resize(records);
        CK(cudaMemcpyAsync(S.phaseHost.data(), S.phaseClock.p, records * sizeof(unsigned long long), cudaMemcpyDeviceToHost, S.stream));
    }
    CK(cudaStreamSynchronize(S.stream));
    if (S.sections) {   // each record's time since the previous record belongs to the phase it closes
        const unsigned long long mask = 0x00FFFFFFFFFFFFFFull;
        unsigned long long last = 0;
        for (size_t i = 0; i < records; i++) {
            unsigned long long r = S.phaseHost[i];
            if (r == 0) continue;
            unsigned tag = (unsigned)(r >> 56);
            unsigned long long ns = r & mask;
            if (last != 0 && tag != kPhaseFrameStart && tag < 8) {
                S.sectionMs[tag] += (double)(ns - last) * 1e-6;
                S.sectionCount[tag]++;
            }
            last = ns;
        }
    }
    if (fc.cut) S.havePrev = true;
    if (S.toolArmed) S.toolFrom = S.tool;
    if (S.hostState[2] != 0u) return LCS_ERR_DEVICE_TIMEOUT;
    S.rotParity = (int)((S.hostState[3] & 1u) ^ (followUp ? 1u : 0u));
    return 0;
}

// Frames again from the post-sever lattice, then the surface rebuild (plugin_api.cpp:157-165); the
// surface itself is not built here.
LCS_API int LCS_Finalize() {
    if (!S.physReady) return -1;
    const int p = S.rotParity;
    particleRotKernel<<<(S.N + 255) / 256, 256, 0, S.stream>>>(deviceMesh(), nullptr, p);
    CK(cudaGetLastError());
    S.rotParity = p ^ 1;
    return buildSurface();
}
// physics_compute_rotations (V/physics.cu:399-411) alone: one particle-frame pass from the current
// lattice, without the surface rebuild LCS_Finalize adds.
LCS_API int GBT_ComputeParticleFrames() {
    if (!S.physReady) return -1;
    const int p = S.rotParity;
    particleRotKernel<<<(S.N + 255) / 256, 256, 0, S.stream>>>(deviceMesh(), nullptr, p);
    CK(cudaGetLastError());
    S.rotParity = p ^ 1;
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
// Surface readback (plugin_api.cpp:84-100): a non-indexed triangle soup, 3 vertices per triangle.
LCS_API int LCS_GetSurfaceCounts(int* vertexCount, int* indexCount) {
    if (!S.surfaceReady) return -1;
    CK(cudaMemcpyAsync(S.hostState + 7, S.triCount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    if (vertexCount) *vertexCount = (int)S.hostState[7];
    if (indexCount) *indexCount = (int)S.hostState[7];
    return 0;
}
LCS_API int LCS_GetSurface(float* outPos3, float* outNrm3, int* outIdx) {
    if (!S.surfaceReady) return -1;
    CK(cudaMemcpyAsync(S.hostState + 7, S.triCount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    const size_t n = S.hostState[7];
    if (outPos3 && n) CK(cudaMemcpyAsync(outPos3, S.outPos.p, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, S.stream));
    if (outNrm3 && n) CK(cudaMemcpyAsync(outNrm3, S.outNrm.p, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    if (outIdx) for (size_t i = 0; i < n; i++) outIdx[i] = (int)i;
    return 0;
}
// Voxel ids of the triangles (3 per triangle, the order of LCS_GetSurface): the indexed form of the
// soup, whose vertex v is voxel v's feature point (recon_tri, V/dc_recon.cu:693).
LCS_API int GBT_GetSurfaceTriangles(int* out3T) {
    if (!S.surfaceReady || !out3T) return -1;
    CK(cudaMemcpyAsync(S.hostState + 7, S.triCount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    const size_t n = S.hostState[7];
    if (n) CK(cudaMemcpyAsync(out3T, S.tri.p, n * sizeof(int), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int LCS_GetSurfaceAux(float* outAux4) {
    if (!S.surfaceReady || !outAux4) return -1;
    CK(cudaMemcpyAsync(S.hostState + 7, S.triCount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    const size_t n = S.hostState[7];
    if (n) CK(cudaMemcpyAsync(outAux4, S.outAux.p, n * sizeof(float4), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int GBT_GetParticleRot(float* out9) {
    if (!S.physReady || !out9) return -1;
    CK(cudaMemcpyAsync(out9, S.rotParity ? S.rotB.p : S.rotA.p, (size_t)9 * S.N * sizeof(float), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API void* GBT_ParticleRotDevice() { return S.physReady ? (void*)(S.rotParity ? S.rotB.p : S.rotA.p) : nullptr; }

// ---------------------------------------------------------------------------------------------
// readback
// ---------------------------------------------------------------------------------------------
// xyz of the N node records into the caller's 3N floats: packed by a kernel, then one copy straight
// into the caller's buffer (no per-call allocation, no host repacking; 0.025 ms for the 135,309
// nodes of the 64x32x48 lattice against 0.12 ms through pinned staging plus a host copy)
static int readNodeXyz(const float4* src, float* out) {
    if (S.packedXyz.n < (size_t)3 * S.N) return -1;
    packXyzKernel<<<(S.N + 255) / 256, 256, 0, S.stream>>>(S.N, src, S.packedXyz.p);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, S.packedXyz.p, (size_t)3 * S.N * sizeof(float), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int LCS_GetCornerPos(float* out) {
    if (!S.reconReady || !out) return -1;
    return readNodeXyz(S.pos.p, out);
}
LCS_API int LCS_GetVelocities(float* out) {
    if (!S.physReady || !out) return -1;
    return readNodeXyz(S.vel.p, out);
}
LCS_API int LCS_GetNbrIdx(int* out) {
    if (!S.physReady || !out) return -1;
    CK(cudaMemcpyAsync(out, S.nbr.p, (size_t)6 * S.N * sizeof(int), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int LCS_GetBendPairs(void* out) {
    if (!S.physReady || !out) return -1;
    CK(cudaMemcpyAsync(out, S.bendPairs.p, S.bendPairs.n * sizeof(BendRecord), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int LCS_GetTopologyRevision(unsigned* revision) {
    if (!revision) return -1;
    if (!S.cutReady) { *revision = 0; return 0; }
    CK(cudaMemcpyAsync(S.hostState + 4, S.counters.p, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    *revision = S.hostState[4];
    return 0;
}
LCS_API int LCS_GetCutEdgeFractions(float* out) {
    if (!S.cutReady || !out) return -1;
    CK(cudaMemcpyAsync(out, S.edgeCutT.p, (size_t)6 * S.N * sizeof(float), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int LCS_GetVoxelCutMask(unsigned* out) {
    if (!S.cutReady || !out) return -1;
    CK(cudaMemcpyAsync(out, S.cutMask.p, S.cutMask.n * sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}
LCS_API int GBT_GetActive(int* outN) {
    if (!S.physReady || !outN) return -1;
    CK(cudaMemcpyAsync(outN, S.active.p, (size_t)S.N * sizeof(int), cudaMemcpyDeviceToHost, S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
}

// Restore of the state one frame carries into the next (the reference keeps it in recon_corner_pos,
// physics_vel, physics_nbr_idx, physics_bend_pairs, physics_active, the cut module's voxel mask,
// edge fractions and topology revision, and physics_particle_rot): a checkpoint taken with the
// getters, or another solver's state to continue from.  Null arguments keep the current values.
// Every table is checked before anything is written, so a rejected call (-1004) changes nothing;
// the liveness flags are derived again at the next frame.
LCS_API int GBT_SetState(const float* pos3N, const float* vel3N, const int* nbr6N, const void* bendPairs, const int* active,
                         const unsigned* cutMaskV, const float* edgeCutT6N, const float* rot9N, int setRevision, unsigned revision) {
    if (!S.physReady) return XPBD_ERR_NOT_READY;
    if ((cutMaskV || edgeCutT6N || setRevision) && !S.cutReady) return XPBD_ERR_BAD_ARG;
    const size_t N = (size_t)S.N;
    for (size_t k = 0; pos3N && k < 3 * N; k++) if (!std::isfinite(pos3N[k])) return XPBD_ERR_BAD_ARG;
    for (size_t k = 0; vel3N && k < 3 * N; k++) if (!std::isfinite(vel3N[k])) return XPBD_ERR_BAD_ARG;
    for (size_t k = 0; rot9N && k < 9 * N; k++) if (!std::isfinite(rot9N[k])) return XPBD_ERR_BAD_ARG;
    for (size_t i = 0; active && i < N; i++) if (active[i] != 0 && active[i] != 1) return XPBD_ERR_BAD_ARG;
    if (nbr6N) {   // a live slot holds the lattice neighbour in its own direction, or -1
        const long long stride[3] = {1, S.dx + 1, (long long)(S.dx + 1) * (S.dy + 1)};
        const int extent[3] = {S.dx, S.dy, S.dz};
        for (size_t i = 0; i < N; i++) {
            const int c[3] = {(int)(i % (S.dx + 1)), (int)(i / (S.dx + 1) % (S.dy + 1)), (int)(i / stride[2])};
            for (int s = 0; s < 6; s++) {
                const int v = nbr6N[6 * i + s], a = s >> 1, to = c[a] + ((s & 1) ? 1 : -1);
                if (v != -1 && (to < 0 || to > extent[a] || v != (long long)i + ((s & 1) ? stride[a] : -stride[a]))) return XPBD_ERR_BAD_ARG;
            }
        }
    }
    if (cutMaskV) for (size_t v = 0; v < S.cutMask.n; v++) if (cutMaskV[v] >> 12) return XPBD_ERR_BAD_ARG;
    std::vector<BendRecord> bends;
    if (bendPairs) {   // only the alive flags may differ from the records the session was built with
        bends.resize(S.bendPairs.n);
        CK(cudaMemcpyAsync(bends.data(), S.bendPairs.p, bends.size() * sizeof(BendRecord), cudaMemcpyDeviceToHost, S.stream));
        CK(cudaStreamSynchronize(S.stream));
        const BendRecord* in = (const BendRecord*)bendPairs;
        for (size_t q = 0; q < bends.size(); q++) {
            BendRecord a = bends[q], b = in[q];
            a.alive = b.alive = 0;
            if (std::memcmp(&a, &b, sizeof(BendRecord)) != 0 || (in[q].alive != 0 && in[q].alive != 1)) return XPBD_ERR_BAD_ARG;
            bends[q].alive = in[q].alive;
        }
    }
    const int grid = (S.N + 255) / 256;
    if (pos3N) {
        CK(cudaMemcpyAsync(S.packedXyz.p, pos3N, 3 * N * sizeof(float), cudaMemcpyHostToDevice, S.stream));
        unpackXyzKernel<<<grid, 256, 0, S.stream>>>(S.N, S.packedXyz.p, S.pos.p);
        CK(cudaGetLastError());
        unpackXyzKernel<<<grid, 256, 0, S.stream>>>(S.N, S.packedXyz.p, S.prev.p);
        CK(cudaGetLastError());
    }
    if (vel3N) {
        CK(cudaStreamSynchronize(S.stream));   // packedXyz is free again
        CK(cudaMemcpyAsync(S.packedXyz.p, vel3N, 3 * N * sizeof(float), cudaMemcpyHostToDevice, S.stream));
        unpackXyzKernel<<<grid, 256, 0, S.stream>>>(S.N, S.packedXyz.p, S.vel.p);
        CK(cudaGetLastError());
    }
    if (nbr6N) CK(cudaMemcpyAsync(S.nbr.p, nbr6N, 6 * N * sizeof(int), cudaMemcpyHostToDevice, S.stream));
    if (bendPairs) CK(cudaMemcpyAsync(S.bendPairs.p, bends.data(), bends.size() * sizeof(BendRecord), cudaMemcpyHostToDevice, S.stream));
    if (active) CK(cudaMemcpyAsync(S.active.p, active, N * sizeof(int), cudaMemcpyHostToDevice, S.stream));
    if (cutMaskV) CK(cudaMemcpyAsync(S.cutMask.p, cutMaskV, S.cutMask.n * sizeof(unsigned), cudaMemcpyHostToDevice, S.stream));
    if (edgeCutT6N) CK(cudaMemcpyAsync(S.edgeCutT.p, edgeCutT6N, 6 * N * sizeof(float), cudaMemcpyHostToDevice, S.stream));
    if (rot9N) CK(cudaMemcpyAsync(S.rotParity ? S.rotB.p : S.rotA.p, rot9N, 9 * N * sizeof(float), cudaMemcpyHostToDevice, S.stream));
    // pageable sources: each copy has taken its bytes when it returns
    if (setRevision) CK(cudaMemcpyAsync(S.counters.p, &revision, sizeof(unsigned), cudaMemcpyHostToDevice, S.stream));
    const unsigned never = ~0u;   // liveness: never derived
    CK(cudaMemcpyAsync(S.state.p, &never, sizeof(unsigned), cudaMemcpyHostToDevice, S.stream));
    S.generation = ++g_sessionGeneration;
    return cudaStatus(cudaStreamSynchronize(S.stream));
}

LCS_API int LCS_GetCutDebug(unsigned* out18, float* alphaOut) {
    if (!S.cutReady || !out18) return -1;
    std::memset(out18, 0, 18 * sizeof(unsigned));
    CK(cudaMemcpyAsync(S.hostState + 4, S.counters.p, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    out18[15] = S.hostState[6];
    out18[16] = S.hostState[5];
    if (alphaOut) *alphaOut = S.cd.cutFPInterp;
    return 0;
}

// ---------------------------------------------------------------------------------------------
// profiling (xpbd_profile_enable/read, xpbd_solver.cu:14-29): device time of each frame launch
// ---------------------------------------------------------------------------------------------
LCS_API void LCS_ProfileEnable(int enabled) {
    for (cudaEvent_t e : S.events) cudaEventDestroy(e);
    S.events.clear();
    S.profile = enabled != 0;
}
LCS_API int LCS_ProfileRead(int steps, float* ms) {
    if (!ms || steps <= 0 || (int)S.events.size() < 2 * steps) return -1;
    CK(cudaEventSynchronize(S.events[2 * steps - 1]));
    float total = 0.f;
    for (int s = 0; s < steps; s++) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, S.events[2 * s], S.events[2 * s + 1]));
        total += t;
    }
    ms[0] = total; ms[1] = 0.f; ms[2] = 0.f;
    return 0;
}
// Section timing (xpbd_profile_sections / _read, xpbd_solver.cu:30-60): while enabled, the first
// CTA stamps the GPU's global timer at the end of every phase of every substep, and the host adds
// each interval to its phase kind.  Read returns "name=ms count=n" lines, or the capacity needed.
LCS_API void LCS_ProfileSections(int enabled) {
    S.sections = enabled != 0;
    for (int k = 0; k < 8; k++) { S.sectionMs[k] = 0.0; S.sectionCount[k] = 0; }
}
LCS_API int LCS_ProfileSectionsRead(char* text, int capacity) {
    static const char* names[8] = {"frame start", "liveness and predict", "edge colours", "bend colours", "tet colours",
                                   "contact and velocity", "ribbon tick", "ribbon tick bricks"};
    std::string out;
    for (int k = 1; k < 8; k++) {
        if (!S.sectionCount[k]) continue;
        char line[160];
        snprintf(line, sizeof line, "%s=%.4f count=%lld\n", names[k], S.sectionMs[k], S.sectionCount[k]);
        out += line;
    }
    if (!text || capacity <= (int)out.size()) return (int)out.size() + 1;
    std::memcpy(text, out.c_str(), out.size() + 1);
    return 0;
}

LCS_API int LCS_SetLaunchMode(int mode) {
    if (mode < 0 || mode > 3) return XPBD_ERR_BAD_ARG;
    S.launchMode = mode;
    return 0;
}
// ---------------------------------------------------------------------------------------------
// Allocation-free step.  Some hosts cannot let a plugin allocate device memory while they run:
// engines and simulators that hand out all GPU memory from their own pool or a fixed budget, and
// real-time loops where a cudaMalloc/cudaFree (which can synchronise the whole device) would stall
// a frame.  LCS_StepNoAlloc advances the session exactly as LCS_Step does, in the shape LCS_Step
// would use, but every piece of frame scratch -- the grid barrier's arrival counter and status
// word, the liveness record, the per-tet compliances of the frame -- lives in the file-scope array
// below, which the driver reserves when the library is loaded and keeps on every GPU that loads it
// until the process exits.  Its size caps the mesh: at most kNoAllocMaxTets tets.
// ---------------------------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocHeaderBytes = 256;                        // state words, 256-byte aligned
constexpr size_t kNoAllocAlphaBytes = (size_t)4 << 20;             // 4 MiB of per-tet compliances
constexpr int kNoAllocMaxTets = (int)(kNoAllocAlphaBytes / sizeof(float2));   // 524,288 tets
static __device__ __align__(256) unsigned char g_stepScratch[kNoAllocHeaderBytes + kNoAllocAlphaBytes];
// Device address of g_stepScratch per device (the symbol itself is only a host-side stand-in),
// looked up by the first LCS_StepNoAlloc of each session (LCS_Init and LCS_Shutdown forget it, so a
// reloaded module after a device reset is looked up again), and the session whose liveness record
// the array holds.
constexpr int kMaxDevices = 64;
unsigned char* g_stepScratchAddr[kMaxDevices] = {};
unsigned long long g_stepScratchOwner[kMaxDevices] = {};
}  // namespace

void forgetStepScratch() {
    for (int d = 0; d < kMaxDevices; d++) { g_stepScratchAddr[d] = nullptr; g_stepScratchOwner[d] = 0; }
}

LCS_API int LCS_StepNoAlloc(float dt) {
    if (!S.physReady) return -1;
    if (S.T > kNoAllocMaxTets) return LCS_ERR_SCRATCH_LIMIT;
    int device = 0;
    CK(cudaGetDevice(&device));
    if (device < 0 || device >= kMaxDevices) return XPBD_ERR_BAD_ARG;
    if (!g_stepScratchAddr[device]) {
        void* address = nullptr;
        CK(cudaGetSymbolAddress(&address, g_stepScratch));
        g_stepScratchAddr[device] = (unsigned char*)address;
        g_stepScratchOwner[device] = 0;
    }
    unsigned char* scratch = g_stepScratchAddr[device];
    unsigned* state = (unsigned*)scratch;
    float2* alpha = (float2*)(scratch + kNoAllocHeaderBytes);

    const int N = S.numSubsteps > 0 ? S.numSubsteps : 1;
    float h = dt / (float)N;
    if (!(h > 0.f) || !std::isfinite(h)) return XPBD_ERR_BAD_DT;
    FrameCoeffs fc = frameCoeffs(h, N);

    // The array keeps whatever the previous call left.  The liveness record (word 0) is kept when
    // this session wrote it and restarts at "never derived" otherwise; the barrier counter, status
    // and frame parity restart at zero; the compliances are written again for this session's tets.
    if (g_stepScratchOwner[device] != S.generation) CK(cudaMemsetAsync(state, 0xFF, sizeof(unsigned), S.stream));
    g_stepScratchOwner[device] = S.generation;
    CK(cudaMemsetAsync(state + 1, 0, 3 * sizeof(unsigned), S.stream));
    if (S.brickCount.p) CK(cudaMemsetAsync(S.brickCount.p, 0, sizeof(unsigned), S.stream));
    if (fc.doStrain) {
        tetAlphaKernel<<<(S.T + 255) / 256, 256, 0, S.stream>>>(S.T, fc.invH2, S.tetStiff.p, alpha);
        CK(cudaGetLastError());
    }
    DeviceMesh m = deviceMesh();
    m.tetAlpha = alpha;
    const Shapes u = usableShapes(fc);
    const int shape = requestedShape(u);   // no timed trials here: they would create events
    bool followUp = false;
    int rc = launchShape(shape, u, fc, m, state, &followUp);
    S.lastFrameBlocks = 0;   // its barrier counter lives in the static scratch, not the session state
    if (rc) return rc;
    unsigned words[2] = {0u, 0u};   // status, current particle-frame buffer
    CK(cudaMemcpyAsync(words, state + 2, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    if (fc.cut) S.havePrev = true;
    if (S.toolArmed) S.toolFrom = S.tool;
    if (words[0] != 0u) return LCS_ERR_DEVICE_TIMEOUT;
    S.rotParity = (int)((words[1] & 1u) ^ (followUp ? 1u : 0u));
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Entry points of the reference's unified contact/grasp/scissors solver (plugin_api.cpp:30-58,
// 202-226, 245-261), which this library does not provide.  The reference adapter
// (endoscopic_tissue/native_backend.py:229-263) binds every one of them and checks the three
// record sizes, so they are exported: the sizes are the reference's record layouts
// (XpbdBladeState 52 B, XpbdScissorsState 244 B, XpbdScissorsResult 124 B, xpbd_solver.h:464-477)
// and every other call returns LCS_ERR_UNSUPPORTED without touching the session.
// ---------------------------------------------------------------------------------------------
LCS_API int LCS_PressureBladeAbiVersion() { return 52; }
LCS_API int LCS_ScissorsAbiVersion() { return 244; }
LCS_API int LCS_ScissorsResultAbiVersion() { return 124; }
LCS_API int LCS_SetPressureBlade(const void*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetPressureBlade(float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetScissors(const void*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetScissors(void*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetScissorsLoads(float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetScissorsWrist(float, float, float) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetJawGeometry(const float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetKnifeGeometry(int, const float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_KnifeBodyDepth(float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_RefineContactSurface(int) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SurfaceDepth(float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetGraspPatch(float, float, float) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetToolDynamics(float, float, float, float) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetJawDynamics(float, float, float, float) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_SetInstrumentControl(int) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetGraspCoreFlags(int, int*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetSolvedTool(float*, float*, int*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetSolvedJaw(float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetContactReaction(float*, int*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetJawLoad(float*) { return LCS_ERR_UNSUPPORTED; }
LCS_API int LCS_GetMaterialQuality(float*) { return LCS_ERR_UNSUPPORTED; }

// Debug builds (GBT_DEBUG_BOUNDS): the session's out-of-range gather record -- violations since the
// last read, the first bad index and its site (BoundsSite) -- then cleared.  Release builds record
// nothing and answer LCS_ERR_UNSUPPORTED.
LCS_API int GBT_DebugBoundsRead(unsigned* out3) {
#ifdef GBT_DEBUG_BOUNDS
    if (!S.physReady || !out3 || !S.bounds.p) return XPBD_ERR_BAD_ARG;
    CK(cudaMemcpyAsync(out3, S.bounds.p, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaMemsetAsync(S.bounds.p, 0, 3 * sizeof(unsigned), S.stream));
    return cudaStatus(cudaStreamSynchronize(S.stream));
#else
    (void)out3;
    return LCS_ERR_UNSUPPORTED;
#endif
}

LCS_API int LCS_SetBarrierTest(int extraArrivals, float budgetSeconds) {
    if (extraArrivals < 0 || !(budgetSeconds > 0.f) || budgetSeconds > 10.f) return XPBD_ERR_BAD_ARG;
    S.syncTestExtra = extraArrivals;
    S.syncBudgetSeconds = budgetSeconds;
    return 0;
}
// Grid barriers the last LCS_Step frame executed (its arrival counter over its CTAs), when that
// frame ran on the whole-GPU grid; the section a barrier closes is one phase of the frame.
LCS_API int GBT_FrameBarriers(unsigned* barriers) {
    if (!barriers) return XPBD_ERR_BAD_ARG;
    if (!S.physReady || S.lastFrameBlocks <= 0) return XPBD_ERR_NOT_READY;
    CK(cudaMemcpyAsync(S.hostState + 5, S.state.p + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    *barriers = S.hostState[5] / (unsigned)S.lastFrameBlocks;
    return 0;
}

// Latency of this library's grid barrier alone: one cooperative launch of the whole-GPU frame
// kernel's grid doing `barriers` barriers and nothing else, timed with CUDA events on the session
// stream (the launch itself included, amortised over the barriers).
LCS_API int GBT_GridBarrierFloor(int barriers, float* usPerBarrier) {
    if (!usPerBarrier || barriers < 1 || barriers > 1000000) return XPBD_ERR_BAD_ARG;
    if (!S.physReady) return XPBD_ERR_NOT_READY;
    if (!S.floorSync.p) CK(S.floorSync.alloc(2));
    CK(cudaMemsetAsync(S.floorSync.p, 0, 2 * sizeof(unsigned), S.stream));
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]));
    CK(cudaEventCreate(&ev[1]));
    unsigned* sync = S.floorSync.p;
    int n = barriers;
    long long budget = (long long)((double)S.syncBudgetSeconds * 1e3 * S.clockKHz);
    void* args[] = {&sync, &n, &budget};
    cudaError_t e = cudaEventRecord(ev[0], S.stream);
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void*)barrierFloorKernel, dim3(S.gridBlocks), dim3(kFrameThreads), args, 0, S.stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], S.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(S.hostState + 5, sync + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S.stream);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (e != cudaSuccess) return -(int)e;
    if (S.hostState[5] != 0u) return LCS_ERR_DEVICE_TIMEOUT;
    *usPerBarrier = 1e3f * ms / (float)barriers;
    return 0;
}

LCS_API void LCS_Shutdown() {
    if (S.stream) cudaStreamSynchronize(S.stream);
    LCS_ProfileEnable(0);
    freeAll();
    forgetStepScratch();
}

// ---------------------------------------------------------------------------------------------
// session view for the differentiable rollout (adjoint_api.cu)
// ---------------------------------------------------------------------------------------------
int gbt::sessionView(SessionView* v) {
    if (!S.physReady || !v) return XPBD_ERR_NOT_READY;
    v->mesh = deviceMesh();
    v->stream = S.stream; v->device = S.device; v->smCount = S.smCount; v->clockKHz = S.clockKHz; v->launchMode = S.launchMode;
    v->N = S.N; v->E = S.E; v->T = S.T; v->numSubsteps = S.numSubsteps > 0 ? S.numSubsteps : 1;
    v->ks = S.ks; v->betaS = S.betaS; v->kb = (S.B > 0) ? S.kb : 0.f; v->strainDamping = S.strainDamping; v->omega = S.omega;
    v->damping = S.damping; v->alpha = S.alpha; v->youngE = S.youngE; v->syncBudgetSeconds = S.syncBudgetSeconds;
    v->cutActive = S.cutReady && S.toolSet && !S.pressure;
    v->volumePasses = S.volumePasses;
    v->contactModel = S.contactModel;
    v->cp = S.cp;
    v->tetColorOrder = S.tetColorOrder.data();
    v->state = S.state.p;
    v->generation = S.generation;
    v->revision = S.cutReady ? S.counters.p : nullptr;
    return 0;
}
