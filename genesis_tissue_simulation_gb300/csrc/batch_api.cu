// Batched tissue instances: many independent meshes of uneven size advanced by one persistent launch
// per frame over a packed instance table.  No counterpart in the reference, which runs one global
// session per process (endoscopic_tissue/native_backend.py:213-218).
//
// Every instance gets exactly the topology of its own plain session (mesh_build.h: the reference's
// greedy colourings), so a batched instance evolves bit for bit as it would alone.  The packed
// table stores colour c of every instance together (colour-major, instances in table order), which
// gives two ways to run a frame, picked by GBT_BatchAutotune:
//   lockstep   all instances advance colour by colour in one cooperative grid (frameKernelLockstep);
//   instances  one CTA per instance at a time, longest-processing-time packing over the CTAs, with
//              only __syncthreads between colours (frameKernelInstances<256|512>).
// GBT_BatchStepMany advances several frames with one CUDA graph launch: the instrument frames of all
// substeps are evaluated on the host (contactFrame, the same operations as on the device), uploaded
// once, and the frame launches are replayed from a captured graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "frame_kernels.h"
#include "mesh_build.h"
#include "../../include/gbtissue.h"

using namespace gbt;

namespace {

template <class T> struct Buf {
    T* p = nullptr; size_t n = 0;
    cudaError_t alloc(size_t count) { release(); n = count; return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)); }
    cudaError_t upload(const T* h, size_t count, cudaStream_t s) {
        cudaError_t e = alloc(count);
        if (e == cudaSuccess && count) e = cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

struct Batch {
    cudaStream_t stream = nullptr;
    int device = 0, smCount = 0, gridBlocks = 0, clockKHz = 2000000;
    bool ready = false;
    int count = 0, N = 0, E = 0, B = 0, T = 0;
    int numSubsteps = 10;
    float ks = 0, kb = 0, alpha = 0, betaS = 0, betaB = 0, youngE = 0, poisson = 0.45f, strainDamping = 0;
    int nEdgeColors = 0, nBendColors = 0, nTetColors = 0;
    std::vector<int> nodeBase, nodeCount, tetCount, edgeCount;
    float typeB[6][9];
    Buf<float4> pos, prev, vel, ext;
    Buf<int> pinned, active, nbr, edgeOwner, edgeLive, bendSrc, bendLive, tetMeta, tetOwner, edgeSupport, nodeInstance;
    Buf<int2> edgeEnds, unionEdge, unionBend, unionTet, instEdge, instBend, instTet;
    Buf<float> edgeRest;
    Buf<int4> bendIJK, tetIds;
    Buf<BendRecord> bendPairs;
    Buf<float2> tetStiff, tetAlpha;
    Buf<int> nodeBaseD, nodeCountD, order, ctaStart;
    Buf<unsigned> derived, state;
    Buf<unsigned> bounds;                            // debug builds: out-of-range gather record
    // implicit lattice elements (tissue_device.cuh): codes in colour order, per-instance geometry,
    // per-instance per-type stiffness and compliances; `useCodes` selects them over the explicit tables
    Buf<unsigned> tetCode, edgeCode; Buf<int4> instGeo; Buf<float2> instStiff, instAlpha;
    bool codesAvailable = false, useCodes = false;
    Buf<int> mobile;                                 // nodes of positive inverse mass (lockstep node passes)
    Buf<ContactFrame> frames;
    unsigned* hostStatus = nullptr;
    ContactFrame* framesHost = nullptr; size_t framesHostCap = 0;
    Buf<float> packedXyz;                             // GBT_BatchGetPositions: xyz packed on the device (3N)
    // instruments
    std::vector<ToolPose> toolFrom, tool;
    bool armed = false;
    ContactParams cp{0.02f, 1.0e-7f, 0.5f, 0.045f, 0.25f};
    float lastH = -1.f;
    // launch
    int mode = 0, threads = 256, ctas = 0;            // mode 0 lockstep grid, 1 one CTA per instance, 2 clusters
    int packing = 0;                                  // modes 1, 2: how instances are dealt to CTAs / clusters (packInstances)
    struct Trial { int mode, threads, packing, tables; float ms; };
    std::vector<Trial> trials;                        // the last autotune's table
    int clusterLogK = 1, clusterSlots = 0;            // mode 2: CTAs per cluster (2^logK), shared-memory slots per CTA
    cudaGraphExec_t graph = nullptr; int graphSteps = 0; int graphMode = -1; float graphDt = 0.f;
    bool profile = false; std::vector<cudaEvent_t> events;
};
Batch G;

#define CK(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) return -(int)_e; } while (0)

void dropGraph() { if (G.graph) cudaGraphExecDestroy(G.graph); G.graph = nullptr; G.graphSteps = 0; }

void releaseAll() {
    dropGraph();
    for (auto* b : {&G.pos, &G.prev, &G.vel, &G.ext}) b->release();
    for (auto* b : {&G.pinned, &G.active, &G.nbr, &G.edgeOwner, &G.edgeLive, &G.bendSrc, &G.bendLive, &G.tetMeta, &G.tetOwner,
                    &G.edgeSupport, &G.nodeInstance, &G.nodeBaseD, &G.nodeCountD, &G.order, &G.ctaStart}) b->release();
    for (auto* b : {&G.edgeEnds, &G.unionEdge, &G.unionBend, &G.unionTet, &G.instEdge, &G.instBend, &G.instTet}) b->release();
    G.edgeRest.release(); G.bendIJK.release(); G.tetIds.release(); G.bendPairs.release(); G.tetStiff.release(); G.tetAlpha.release();
    G.derived.release(); G.state.release(); G.frames.release(); G.bounds.release();
    G.tetCode.release(); G.edgeCode.release(); G.instGeo.release(); G.instStiff.release(); G.instAlpha.release();
    G.codesAvailable = G.useCodes = false;
    G.mobile.release();
    if (G.framesHost) cudaFreeHost(G.framesHost);
    G.framesHost = nullptr; G.framesHostCap = 0;
    G.packedXyz.release();
    for (cudaEvent_t e : G.events) cudaEventDestroy(e);
    G.events.clear();
    G.ready = false; G.armed = false; G.lastH = -1.f;
    G.packing = 0; G.trials.clear();
}

int ensureDevice() {
    if (G.stream) return 0;
    CK(cudaGetDevice(&G.device));
    CK(cudaDeviceGetAttribute(&G.smCount, cudaDevAttrMultiProcessorCount, G.device));
    int khz = 0;
    if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, G.device) == cudaSuccess && khz > 0) G.clockKHz = khz;
    CK(cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking));
    CK(cudaMallocHost(&G.hostStatus, 4 * sizeof(unsigned)));
    int perSm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, frameKernelLockstep, kFrameThreads, 0));
    G.gridBlocks = std::max(1, perSm) * G.smCount;
    return 0;
}

// Instances dealt to `ctas` CTAs (or clusters), by G.packing:
//   0  longest processing time first on tet counts (the heaviest instance to the least loaded CTA);
//   1  the same on a work estimate that counts every element a frame sweeps (tets + edges + nodes);
//   2  instances in decreasing size dealt round-robin in serpentine order (no load accounting).
// Every packing gives the same results: an instance is advanced by one CTA or cluster either way.
int packInstances(int ctas) {
    ctas = std::max(1, std::min(ctas, G.count));
    auto work = [](int i) -> long long {
        return G.packing == 1 ? (long long)G.tetCount[i] + G.edgeCount[i] + G.nodeCount[i] : (long long)G.tetCount[i];
    };
    std::vector<int> byWork(G.count);
    std::iota(byWork.begin(), byWork.end(), 0);
    std::stable_sort(byWork.begin(), byWork.end(), [&](int a, int b) { return work(a) > work(b); });
    std::vector<long long> load(ctas, 0);
    std::vector<std::vector<int>> lists(ctas);
    for (size_t k = 0; k < byWork.size(); k++) {
        const int i = byWork[k];
        int best;
        if (G.packing == 2) {
            const int lap = (int)(k / ctas), at = (int)(k % ctas);
            best = (lap & 1) ? ctas - 1 - at : at;
        } else {
            best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        }
        lists[best].push_back(i);
        load[best] += work(i) + 1;
    }
    std::vector<int> order, start(1, 0);
    for (auto& l : lists) { order.insert(order.end(), l.begin(), l.end()); start.push_back((int)order.size()); }
    CK(G.order.upload(order.data(), order.size(), G.stream));
    CK(G.ctaStart.upload(start.data(), start.size(), G.stream));
    G.ctas = ctas;
    return 0;
}

DeviceMesh batchMesh() {
    DeviceMesh m{};
    m.nNodes = G.N; m.nodeBase = 0; m.dx = m.dy = m.dz = 0;
    m.pos = G.pos.p; m.prev = G.prev.p; m.vel = G.vel.p; m.ext = G.ext.p;
    m.pinned = G.pinned.p; m.active = G.active.p; m.nbr = G.nbr.p;
    m.nEdgeColors = G.nEdgeColors; m.edgeRange = G.unionEdge.p;
    m.edgeEnds = G.edgeEnds.p; m.edgeRest = G.edgeRest.p; m.edgeOwner = G.edgeOwner.p; m.edgeLive = G.edgeLive.p;
    m.nBendColors = G.nBendColors; m.bendRange = G.unionBend.p;
    m.bendIJK = G.bendIJK.p; m.bendSrc = G.bendSrc.p; m.bendLive = G.bendLive.p; m.bendPairs = G.bendPairs.p; m.nBendPairs = (int)G.bendPairs.n;
    m.nTetColors = G.nTetColors; m.tetRange = G.unionTet.p;
    m.tetIds = G.tetIds.p; m.tetMeta = G.tetMeta.p; m.tetOwner = G.tetOwner.p; m.tetAlpha = G.tetAlpha.p; m.tetStiff = G.tetStiff.p;
    m.edgeSupport = G.edgeSupport.p;
    m.nodeInstance = G.nodeInstance.p; m.contactFrames = G.frames.p; m.nInstances = G.count;
    std::memcpy(m.typeB, G.typeB, sizeof(G.typeB));
    m.bounds = G.bounds.p;
    if (G.useCodes) { m.tetCode = G.tetCode.p; m.edgeCode = G.edgeCode.p; m.instGeo = G.instGeo.p; m.instAlpha = G.instAlpha.p; }
    if (G.mode == 0) { m.mobile = G.mobile.p; m.nMobile = (int)G.mobile.n; }   // the per-instance shapes sweep their ranges
    return m;
}

FrameCoeffs frameCoeffs(float h) {
    FrameCoeffs fc{};
    const int N = G.numSubsteps;
    fc.numSubsteps = N; fc.substeps = N; fc.firstSubstep = 0;
    float at = G.ks > 0.f ? 1.f / (G.ks * h * h) : 0.f;
    fc.velScale = 1.f / (1.f + G.alpha * h);
    fc.betaGammaHS = at * G.betaS * h;
    fc.alphaTilde = at;
    fc.doBend = (G.B > 0 && G.kb > 0.f) ? 1 : 0;
    fc.alphaB = fc.doBend ? 1.f / (G.kb * h * h) : 0.f;
    fc.betaGammaHB = fc.alphaB * G.betaB * h;
    fc.h = h; fc.invH = 1.f / h; fc.invH2 = 1.f / (h * h);
    fc.doStrain = (G.T > 0 && G.youngE > 0.f) ? 1 : 0;
    fc.fallback = (fc.doStrain && G.ks <= 0.f) ? 1 : 0;
    fc.doEdges = (G.ks > 0.f || fc.fallback) ? 1 : 0;
    fc.fallbackInvEh2 = fc.fallback ? 1.f / (G.youngE * h * h) : 0.f;
    fc.perpDamp = G.betaS > 0.f ? 1 : 0;
    fc.betaS = G.betaS;
    fc.omega = 1.f;
    fc.dampingOverH = fmaxf(0.f, G.strainDamping) / h;
    fc.invScale = 1.f / (1.f + fc.dampingOverH); fc.invBulkScale = fc.invScale;
    fc.contact = G.armed ? 1 : 0;
    fc.contactAlphaH2 = G.cp.contactAlpha / (h * h);
    fc.spinBudget = (long long)(2.0 * 1e3 * G.clockKHz);
    return fc;
}

int ensureFramesHost(size_t records) {
    if (records <= G.framesHostCap) return 0;
    if (G.framesHost) cudaFreeHost(G.framesHost);
    G.framesHost = nullptr;
    CK(cudaMallocHost(&G.framesHost, records * sizeof(ContactFrame)));
    G.framesHostCap = records;
    return 0;
}

// Instrument frames of `steps` frames into the pinned staging area, with the single session's command
// semantics (xpbd_set_tool, xpbd_solver.cu:2327-2334, 3467-3483): a new command for frame k makes the
// previous command its starting pose (itself when no instrument was armed yet); the frame
// interpolates from it; after the frame the starting pose is the command.
void stageFrames(int steps, const ToolPose* tools, float h) {
    const int NS = G.numSubsteps;
    float alpha = G.cp.contactAlpha / (h * h);
    std::vector<ToolPose> from = G.toolFrom, to = G.tool;
    bool armed = G.armed;
    for (int k = 0; k < steps; k++) {
        if (tools) {
            std::vector<ToolPose> next(tools + (size_t)k * G.count, tools + (size_t)(k + 1) * G.count);
            from = armed ? to : next;
            to = next;
            armed = true;
        }
        for (int s = 0; s < NS; s++) {
            float t = fminf(1.f, (float)(s + 1) / (float)NS);
            for (int i = 0; i < G.count; i++)
                G.framesHost[((size_t)k * NS + s) * G.count + i] = contactFrame(from[i], to[i], t, G.cp, alpha);
        }
        from = to;
    }
    G.tool = to;
    G.toolFrom = to;
    G.armed = armed;
}

int launchFrame(const FrameCoeffs& fc, const ContactFrame* frames) {
    DeviceMesh m = batchMesh();
    m.contactFrames = frames;
    if (G.mode == 0) {
        CutParams cu{};
        ToolPose none{};
        ContactParams cp = G.cp;
        unsigned* state = G.state.p;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(G.gridBlocks); cfg.blockDim = dim3(kFrameThreads); cfg.stream = G.stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative; attr[0].val.cooperative = 1;
        cfg.attrs = attr; cfg.numAttrs = 1;
        CK(cudaMemsetAsync(state + 1, 0, sizeof(unsigned), G.stream));
        CK(cudaLaunchKernelEx(&cfg, frameKernelLockstep, m, fc, none, none, cp, cu, state));
    } else if (G.mode == 1) {
        InstanceTable it{G.nodeBaseD.p, G.nodeCountD.p, G.instEdge.p, G.instBend.p, G.instTet.p, G.order.p, G.ctaStart.p, G.derived.p};
        if (G.threads == 512) frameKernelInstances512<<<G.ctas, 512, 0, G.stream>>>(m, fc, G.cp, it);
        else frameKernelInstances256<<<G.ctas, 256, 0, G.stream>>>(m, fc, G.cp, it);
        CK(cudaGetLastError());
    } else {
        InstanceTable it{G.nodeBaseD.p, G.nodeCountD.p, G.instEdge.p, G.instBend.p, G.instTet.p, G.order.p, G.ctaStart.p, G.derived.p};
        const int K = 1 << G.clusterLogK;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(G.ctas * K); cfg.blockDim = dim3(kClusterThreads); cfg.stream = G.stream;
        cfg.dynamicSmemBytes = (size_t)G.clusterSlots * sizeof(float4);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = K; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr; cfg.numAttrs = 1;
        ContactParams cp = G.cp;
        int logK = G.clusterLogK;
        CK(cudaLaunchKernelEx(&cfg, frameKernelCluster, m, fc, cp, it, logK));
    }
    return 0;
}

// Cluster launch shape for K CTAs per cluster: the shared-memory slots of the largest instance
// (interleaved in blocks of kClusterThreads nodes over the K CTAs), the number of clusters that
// fit on the GPU at once, and the LPT packing of the instances over those clusters.
int packClusters(int K) {
    int logK = 0;
    while ((1 << logK) < K) logK++;
    const int block = kClusterThreads * K;
    int slots = 0;
    for (int i = 0; i < G.count; i++) slots = std::max(slots, ((G.nodeCount[i] + block - 1) / block) * kClusterThreads);
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, G.device));
    const size_t bytes = (size_t)slots * sizeof(float4);
    if (bytes + 1024 > (size_t)optin) return LCS_ERR_UNSUPPORTED;   // an instance does not fit this cluster size
    CK(cudaFuncSetAttribute((const void*)frameKernelCluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(K); cfg.blockDim = dim3(kClusterThreads); cfg.dynamicSmemBytes = bytes;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr; cfg.numAttrs = 1;
    int clusters = 0;
    CK(cudaOccupancyMaxActiveClusters(&clusters, (const void*)frameKernelCluster, &cfg));
    if (clusters <= 0) return LCS_ERR_UNSUPPORTED;
    G.clusterLogK = logK;
    G.clusterSlots = slots;
    return packInstances(clusters);
}

int prepareAlphas(float h) {
    if (G.T > 0 && G.youngE > 0.f && h != G.lastH) {
        tetAlphaKernel<<<(G.T + 255) / 256, 256, 0, G.stream>>>(G.T, 1.f / (h * h), G.tetStiff.p, G.tetAlpha.p);
        CK(cudaGetLastError());
        if (G.codesAvailable) {   // the same operation on each instance's six Kuhn types
            tetAlphaKernel<<<(6 * G.count + 255) / 256, 256, 0, G.stream>>>(6 * G.count, 1.f / (h * h), G.instStiff.p, G.instAlpha.p);
            CK(cudaGetLastError());
        }
        G.lastH = h;
    }
    return 0;
}

// Advance `steps` frames; `tools` is [steps][count] XpbdToolState or null (instruments unchanged).
int stepFrames(float dt, int steps, const ToolPose* tools, bool useGraph) {
    if (!G.ready) return XPBD_ERR_NOT_READY;
    if (steps <= 0) return XPBD_ERR_BAD_ARG;
    float h = dt / (float)G.numSubsteps;
    if (!(h > 0.f) || !std::isfinite(h)) return XPBD_ERR_BAD_DT;
    int rc = prepareAlphas(h);
    if (rc) return rc;
    const size_t per = (size_t)G.numSubsteps * G.count;
    rc = ensureFramesHost(per * steps);
    if (rc) return rc;
    bool contact = G.armed || tools;
    if (contact) stageFrames(steps, tools, h);
    FrameCoeffs fc = frameCoeffs(h);
    if (G.frames.n < per * steps) { CK(G.frames.alloc(per * steps)); dropGraph(); }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (G.profile) { CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1)); CK(cudaEventRecord(e0, G.stream)); }
    CK(cudaMemsetAsync(G.state.p + 2, 0, sizeof(unsigned), G.stream));
    if (useGraph) {
        if (G.graph && (G.graphSteps != steps || G.graphMode != G.mode * 1000 + G.threads + (fc.contact ? 1 : 0) || G.graphDt != dt)) dropGraph();
        if (!G.graph) {
            CK(cudaStreamBeginCapture(G.stream, cudaStreamCaptureModeThreadLocal));
            CK(cudaMemcpyAsync(G.frames.p, G.framesHost, per * steps * sizeof(ContactFrame), cudaMemcpyHostToDevice, G.stream));
            for (int k = 0; k < steps && rc == 0; k++) rc = launchFrame(fc, G.frames.p + per * k);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(G.stream, &g);
            if (rc) { if (g) cudaGraphDestroy(g); return rc; }
            if (e != cudaSuccess) return -(int)e;
            e = cudaGraphInstantiate(&G.graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return -(int)e;
            G.graphSteps = steps; G.graphMode = G.mode * 1000 + G.threads + (fc.contact ? 1 : 0); G.graphDt = dt;
        }
        CK(cudaGraphLaunch(G.graph, G.stream));
    } else {
        if (contact) CK(cudaMemcpyAsync(G.frames.p, G.framesHost, per * steps * sizeof(ContactFrame), cudaMemcpyHostToDevice, G.stream));
        for (int k = 0; k < steps; k++) {
            rc = launchFrame(fc, G.frames.p + per * k);
            if (rc) return rc;
        }
    }
    if (G.profile) { CK(cudaEventRecord(e1, G.stream)); G.events.push_back(e0); G.events.push_back(e1); }
    CK(cudaMemcpyAsync(G.hostStatus, G.state.p + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, G.stream));
    CK(cudaStreamSynchronize(G.stream));
    return G.hostStatus[0] != 0u ? LCS_ERR_DEVICE_TIMEOUT : 0;
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
LCS_API int GBT_BatchInit(int count, const GbtInstanceDesc* inst, const GbtBatchParams* params) {
    releaseAll();
    if (count <= 0 || !inst || !params) return XPBD_ERR_BAD_ARG;
    if (!std::isfinite(params->youngE) || params->youngE < 0.f || !std::isfinite(params->poisson) || params->poisson < 0.f ||
        params->poisson >= 0.5f || !std::isfinite(params->strainDamping) || params->strainDamping < 0.f) return -2004;
    int rc = ensureDevice();
    if (rc) return rc;
    G.N = G.E = G.B = G.T = 0;
    G.nEdgeColors = G.nBendColors = G.nTetColors = 0;
    G.mode = 0; G.threads = 256;
    G.count = count;
    G.numSubsteps = params->substeps > 0 ? params->substeps : 20;
    G.ks = params->ks; G.kb = params->kb; G.alpha = params->alpha; G.betaS = params->cs; G.betaB = params->cb;
    G.youngE = params->youngE; G.poisson = params->poisson; G.strainDamping = params->strainDamping;
    std::vector<HostMesh> meshes(count);
    for (int i = 0; i < count; i++) {
        const GbtInstanceDesc& d = inst[i];
        if (d.dimsX <= 0 || d.dimsY <= 0 || d.dimsZ <= 0 || !d.cornerPos || !d.mass || !d.pinned || !d.active || !d.nbrIdx ||
            !d.restNbr || d.bendPairCount < 0 || (d.bendPairCount > 0 && !d.bendPairs)) return XPBD_ERR_BAD_ARG;
        int n = (d.dimsX + 1) * (d.dimsY + 1) * (d.dimsZ + 1);
        std::vector<float> zeros(3 * (size_t)n, 0.f);
        MeshInput in{d.dimsX, d.dimsY, d.dimsZ, d.cornerPos, d.mass, d.pinned, d.active, zeros.data(), d.nbrIdx, d.restNbr,
                     d.bendPairs, d.bendPairCount, G.youngE, G.poisson};
        rc = buildHostMesh(in, meshes[i]);
        if (rc) return rc;
        HostMesh& hm = meshes[i];
        if (d.tetMuV && d.tetKappaV)   // per-tet material in storage order, placed through the colour order
            for (int k = 0; k < hm.T; k++) {
                int t = hm.tetColorOrder[k];
                if (!(d.tetMuV[t] > 0.f) || !(d.tetKappaV[t] > 0.f)) return XPBD_ERR_BAD_ARG;
                hm.tetStiff[k] = make_float2(d.tetMuV[t], d.tetKappaV[t]);
            }
        if (d.stiffnessScale > 0.f && d.stiffnessScale != 1.f) {
            if (!std::isfinite(d.stiffnessScale)) return XPBD_ERR_BAD_ARG;
            for (auto& s : hm.tetStiff) s = make_float2(s.x * d.stiffnessScale, s.y * d.stiffnessScale);
        }
        for (int a = 0; a < 54; a++)   // one rest shape per Kuhn type for the whole table
            if (std::fabs((&hm.typeB[0][0])[a] - (&meshes[0].typeB[0][0])[a]) > 1e-6f * (1.f + std::fabs((&meshes[0].typeB[0][0])[a])))
                return XPBD_ERR_IRREGULAR_REST;
    }
    std::memcpy(G.typeB, meshes[0].typeB, sizeof(G.typeB));
    // instance offsets and colour counts
    G.nodeBase.assign(count, 0); G.nodeCount.assign(count, 0); G.tetCount.assign(count, 0); G.edgeCount.assign(count, 0);
    int bendPairBase = 0;
    std::vector<int> bendBase(count);
    for (int i = 0; i < count; i++) {
        G.nodeBase[i] = G.N; G.nodeCount[i] = meshes[i].N; G.tetCount[i] = meshes[i].T; G.edgeCount[i] = meshes[i].E;
        G.N += meshes[i].N; G.E += meshes[i].E; G.B += meshes[i].B; G.T += meshes[i].T;
        bendBase[i] = bendPairBase; bendPairBase += inst[i].bendPairCount;
        G.nEdgeColors = std::max(G.nEdgeColors, (int)meshes[i].edgeColorOff.size() - 1);
        G.nBendColors = std::max(G.nBendColors, (int)meshes[i].bendColorOff.size() - 1);
        G.nTetColors = std::max(G.nTetColors, (int)meshes[i].tetColorOff.size() - 1);
    }
    // node arrays and topology, instance after instance
    std::vector<float4> pos, ext; std::vector<int> pinned, active, nbr, nodeInst;
    std::vector<BendRecord> bends;
    pos.reserve(G.N); ext.reserve(G.N);
    for (int i = 0; i < count; i++) {
        const HostMesh& hm = meshes[i];
        const int base = G.nodeBase[i];
        pos.insert(pos.end(), hm.pos.begin(), hm.pos.end());
        ext.insert(ext.end(), hm.ext.begin(), hm.ext.end());
        pinned.insert(pinned.end(), inst[i].pinned, inst[i].pinned + hm.N);
        active.insert(active.end(), inst[i].active, inst[i].active + hm.N);
        for (int k = 0; k < 6 * hm.N; k++) nbr.push_back(inst[i].nbrIdx[k] >= 0 ? inst[i].nbrIdx[k] + base : -1);
        nodeInst.insert(nodeInst.end(), hm.N, i);
        const BendRecord* bp = (const BendRecord*)inst[i].bendPairs;
        for (int b = 0; b < inst[i].bendPairCount; b++) {
            BendRecord r = bp[b];
            r.i += base; r.j = r.j >= 0 ? r.j + base : r.j; r.k = r.k >= 0 ? r.k + base : r.k;
            bends.push_back(r);
        }
    }
    // colour-major element tables: colour c of instance 0, of instance 1, ...
    std::vector<int2> eEnds, uEdge, uBend, uTet, iEdge((size_t)count * G.nEdgeColors), iBend((size_t)count * G.nBendColors),
        iTet((size_t)count * G.nTetColors);
    std::vector<float> eRest; std::vector<int> eOwner, bSrc, tMeta, tOwner; std::vector<int4> bIJK, tIds; std::vector<float2> tStiff;
    auto colourSlice = [](const std::vector<int>& off, int c) {
        return c + 1 < (int)off.size() ? std::make_pair(off[c], off[c + 1]) : std::make_pair(0, 0);
    };
    for (int c = 0; c < G.nEdgeColors; c++) {
        int lo = (int)eEnds.size();
        for (int i = 0; i < count; i++) {
            const HostMesh& hm = meshes[i];
            const int base = G.nodeBase[i];
            auto sl = colourSlice(hm.edgeColorOff, c);
            iEdge[(size_t)i * G.nEdgeColors + c] = make_int2((int)eEnds.size(), (int)eEnds.size() + sl.second - sl.first);
            for (int k = sl.first; k < sl.second; k++) {
                eEnds.push_back(make_int2(hm.edgeEnds[k].x + base, hm.edgeEnds[k].y + base));
                eRest.push_back(hm.edgeRest[k]);
                eOwner.push_back(hm.edgeOwner[k] + 6 * base);
            }
        }
        uEdge.push_back(make_int2(lo, (int)eEnds.size()));
    }
    for (int c = 0; c < G.nBendColors; c++) {
        int lo = (int)bIJK.size();
        for (int i = 0; i < count; i++) {
            const HostMesh& hm = meshes[i];
            const int base = G.nodeBase[i];
            auto sl = colourSlice(hm.bendColorOff, c);
            iBend[(size_t)i * G.nBendColors + c] = make_int2((int)bIJK.size(), (int)bIJK.size() + sl.second - sl.first);
            for (int k = sl.first; k < sl.second; k++) {
                int4 r = hm.bendIJK[k];
                bIJK.push_back(make_int4(r.x + base, r.y + base, r.z + base, r.w));
                bSrc.push_back(hm.bendSrc[k] + bendBase[i]);
            }
        }
        uBend.push_back(make_int2(lo, (int)bIJK.size()));
    }
    for (int c = 0; c < G.nTetColors; c++) {
        int lo = (int)tIds.size();
        for (int i = 0; i < count; i++) {
            const HostMesh& hm = meshes[i];
            const int base = G.nodeBase[i];
            auto sl = colourSlice(hm.tetColorOff, c);
            iTet[(size_t)i * G.nTetColors + c] = make_int2((int)tIds.size(), (int)tIds.size() + sl.second - sl.first);
            for (int k = sl.first; k < sl.second; k++) {
                int4 d = hm.tetIds[k];
                tIds.push_back(make_int4(d.x + base, d.y + base, d.z + base, d.w + base));
                tMeta.push_back(hm.tetMeta[k]);
                for (int o = 0; o < 3; o++) tOwner.push_back(hm.tetOwner[3 * k + o] + 6 * base);
                tStiff.push_back(hm.tetStiff[k]);
            }
        }
        uTet.push_back(make_int2(lo, (int)tIds.size()));
    }
    // Implicit element codes (tissue_device.cuh), when every element is where the lattice formula
    // puts it: instance nodes below 2^15, instances below 2^13, each tet's nodes the Kuhn path of its
    // type from its corner 0, each edge an axis step of its lower end, one stiffness per instance and
    // Kuhn type, and no tet-support fallback (ks > 0).
    std::vector<unsigned> tCode, eCode;
    std::vector<int4> geo(count);
    std::vector<float2> iStiff((size_t)6 * count, make_float2(0.f, 0.f));
    std::vector<char> seenType((size_t)6 * count, 0);
    bool codes = count < (1 << 13) && G.ks > 0.f;
    for (int i = 0; i < count && codes; i++) {
        const int nx = inst[i].dimsX + 1, nxy = (inst[i].dimsX + 1) * (inst[i].dimsY + 1);
        geo[i] = make_int4(G.nodeBase[i], nx, nxy, 0);
        codes = G.nodeCount[i] < (1 << 15);
    }
    if (codes) {
        // the device decodes with kuhnNodes / kuhnOwners; the same functions must give back every
        // tet's explicit nodes and link slots, or the batch keeps the explicit tables
        const std::vector<int>& nodeInstance = nodeInst;
        tCode.resize(tIds.size());
        for (size_t k = 0; k < tIds.size() && codes; k++) {
            const int4 d = tIds[k];
            const int i = nodeInstance[d.x], type = tMeta[k] & 7;
            const int4 g = geo[i];
            const int local = d.x - g.x;
            const int4 want = kuhnNodes(type, d.x, g.y, g.z);
            int own[3];
            kuhnOwners(type, d.x, g.y, g.z, own);
            codes = type < 6 && want.x == d.x && want.y == d.y && want.z == d.z && want.w == d.w &&
                    own[0] == tOwner[3 * k] && own[1] == tOwner[3 * k + 1] && own[2] == tOwner[3 * k + 2];
            float2& st = iStiff[(size_t)6 * i + type];
            if (!seenType[(size_t)6 * i + type]) { st = tStiff[k]; seenType[(size_t)6 * i + type] = 1; }
            codes = codes && std::memcmp(&st, &tStiff[k], sizeof(float2)) == 0;
            tCode[k] = (unsigned)local | (unsigned)type << 15 | kCodeLive | (unsigned)i << 19;
        }
        eCode.resize(eEnds.size());
        for (size_t k = 0; k < eEnds.size() && codes; k++) {
            const int2 d = eEnds[k];
            const int i = nodeInstance[d.x];
            const int4 g = geo[i];
            const int step = d.y - d.x, axis = step == 1 ? 0 : step == g.y ? 1 : step == g.z ? 2 : -1;
            codes = axis >= 0 && eOwner[k] == 6 * d.x + 2 * axis + 1 && nodeInstance[d.y] == i;
            eCode[k] = (unsigned)(d.x - g.x) | (unsigned)(axis & 3) << 15 | kCodeLive | (unsigned)i << 19;
        }
    }
    G.codesAvailable = codes;
    G.useCodes = codes;
    if (codes) {
        CK(G.tetCode.upload(tCode.data(), tCode.size(), G.stream)); CK(G.edgeCode.upload(eCode.data(), eCode.size(), G.stream));
        CK(G.instGeo.upload(geo.data(), count, G.stream)); CK(G.instStiff.upload(iStiff.data(), iStiff.size(), G.stream));
        CK(G.instAlpha.alloc((size_t)6 * count));
    }
    std::vector<float4> zero4(G.N, make_float4(0, 0, 0, 0));
    std::vector<int> ones(std::max(std::max(G.E, G.B), 1), 1), zeros6((size_t)6 * G.N, 0);
    std::vector<unsigned> derived(count, ~0u), state(4, 0u);
    state[0] = ~0u;
    CK(G.pos.upload(pos.data(), G.N, G.stream)); CK(G.prev.upload(pos.data(), G.N, G.stream));
    {   // prev starts equal to pos and vel at zero (below), so a node of inverse mass 0 never changes
        std::vector<int> mob;
        for (int i = 0; i < G.N; i++) if (pos[i].w > 0.f) mob.push_back(i);
        CK(G.mobile.upload(mob.data(), mob.size(), G.stream));
        G.mobile.n = mob.size();
    }
    CK(G.packedXyz.alloc((size_t)3 * G.N));
    CK(G.vel.upload(zero4.data(), G.N, G.stream)); CK(G.ext.upload(ext.data(), G.N, G.stream));
    CK(G.pinned.upload(pinned.data(), G.N, G.stream)); CK(G.active.upload(active.data(), G.N, G.stream));
    CK(G.nbr.upload(nbr.data(), nbr.size(), G.stream)); CK(G.nodeInstance.upload(nodeInst.data(), G.N, G.stream));
    CK(G.edgeEnds.upload(eEnds.data(), eEnds.size(), G.stream)); CK(G.edgeRest.upload(eRest.data(), eRest.size(), G.stream));
    CK(G.edgeOwner.upload(eOwner.data(), eOwner.size(), G.stream)); CK(G.edgeLive.upload(ones.data(), G.E, G.stream));
    CK(G.bendIJK.upload(bIJK.data(), bIJK.size(), G.stream)); CK(G.bendSrc.upload(bSrc.data(), bSrc.size(), G.stream));
    CK(G.bendLive.upload(ones.data(), G.B, G.stream)); CK(G.bendPairs.upload(bends.data(), bends.size(), G.stream));
    CK(G.tetIds.upload(tIds.data(), tIds.size(), G.stream)); CK(G.tetMeta.upload(tMeta.data(), tMeta.size(), G.stream));
    CK(G.tetOwner.upload(tOwner.data(), tOwner.size(), G.stream)); CK(G.tetStiff.upload(tStiff.data(), tStiff.size(), G.stream));
    CK(G.tetAlpha.alloc(G.T)); CK(G.edgeSupport.upload(zeros6.data(), zeros6.size(), G.stream));
    CK(G.unionEdge.upload(uEdge.data(), uEdge.size(), G.stream)); CK(G.unionBend.upload(uBend.data(), uBend.size(), G.stream));
    CK(G.unionTet.upload(uTet.data(), uTet.size(), G.stream));
    CK(G.instEdge.upload(iEdge.data(), iEdge.size(), G.stream)); CK(G.instBend.upload(iBend.data(), iBend.size(), G.stream));
    CK(G.instTet.upload(iTet.data(), iTet.size(), G.stream));
    CK(G.nodeBaseD.upload(G.nodeBase.data(), count, G.stream)); CK(G.nodeCountD.upload(G.nodeCount.data(), count, G.stream));
    CK(G.derived.upload(derived.data(), count, G.stream)); CK(G.state.upload(state.data(), 4, G.stream));
    rc = packInstances(G.smCount * 2);
    if (rc) return rc;
    G.tool.assign(count, ToolPose{}); G.toolFrom = G.tool;
#ifdef GBT_DEBUG_BOUNDS
    CK(G.bounds.alloc(3));
    CK(cudaMemsetAsync(G.bounds.p, 0, 3 * sizeof(unsigned), G.stream));
#endif
    CK(cudaStreamSynchronize(G.stream));
    G.ready = true;
    return 0;
}

LCS_API int GBT_BatchSetGravity(float gx, float gy, float gz) {
    if (!G.ready) return XPBD_ERR_NOT_READY;
    if (!std::isfinite(gx) || !std::isfinite(gy) || !std::isfinite(gz)) return XPBD_ERR_BAD_ARG;
    gravityKernel<<<(G.N + 255) / 256, 256, 0, G.stream>>>(G.N, gx, gy, gz, G.ext.p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(G.stream));
    return 0;
}

// The contact parameters are frame-kernel arguments, so a CUDA graph captured with the previous ones
// is dropped (the next graph step captures again).
LCS_API void GBT_BatchSetGraspParams(const GraspParamsAbi* p) {
    if (!p) return;
    ContactParams c = G.cp;
    c.jawGapClosed = p->jawGapClosed; c.contactAlpha = p->contactAlpha; c.ccdVelThresh = p->ccdVelThresh;
    c.ccdMaxDisp = p->ccdMaxDisp; c.ccdOmega = p->ccdOmega;
    if (std::memcmp(&c, &G.cp, sizeof(c)) != 0) dropGraph();
    G.cp = c;
}

LCS_API int GBT_BatchSetTools(const void* tools) {
    if (!G.ready || !tools) return XPBD_ERR_BAD_ARG;
    const ToolPose* t = (const ToolPose*)tools;
    G.toolFrom = G.armed ? G.tool : std::vector<ToolPose>(t, t + G.count);
    G.tool.assign(t, t + G.count);
    G.armed = true;
    return 0;
}

LCS_API int GBT_BatchStep(float dt) { return stepFrames(dt, 1, nullptr, false); }

LCS_API int GBT_BatchStepMany(float dt, int steps, const void* tools, int useGraph) {
    return stepFrames(dt, steps, (const ToolPose*)tools, useGraph != 0);
}

// Every instance's node positions (3N floats, packed-table order): packed by a kernel, then one
// copy straight into the caller's buffer (no host repacking).
LCS_API int GBT_BatchGetPositions(float* out3N) {
    if (!G.ready || !out3N) return XPBD_ERR_BAD_ARG;
    if (G.packedXyz.n < (size_t)3 * G.N) CK(G.packedXyz.alloc((size_t)3 * G.N));
    packXyzKernel<<<(G.N + 255) / 256, 256, 0, G.stream>>>(G.N, G.pos.p, G.packedXyz.p);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out3N, G.packedXyz.p, (size_t)3 * G.N * sizeof(float), cudaMemcpyDeviceToHost, G.stream));
    CK(cudaStreamSynchronize(G.stream));
    return 0;
}

LCS_API int GBT_BatchInfo(int* counts8) {
    if (!G.ready || !counts8) return XPBD_ERR_BAD_ARG;
    int v[8] = {G.count, G.N, G.E, G.T, G.nEdgeColors, G.nTetColors, G.mode, G.threads};
    std::memcpy(counts8, v, sizeof(v));
    return 0;
}

LCS_API int GBT_BatchNodeRange(int instance, int* base, int* count) {
    if (!G.ready || instance < 0 || instance >= G.count || !base || !count) return XPBD_ERR_BAD_ARG;
    *base = G.nodeBase[instance]; *count = G.nodeCount[instance];
    return 0;
}

// Element tables of the frame kernels: 1 the implicit lattice codes (the default where the batch
// qualifies), 0 the explicit tables; both give identical results.  Returns -4001 when 1 is asked of a
// batch that does not qualify.
LCS_API int GBT_BatchSetElementTables(int implicitCodes) {
    if (!G.ready) return XPBD_ERR_NOT_READY;
    if (implicitCodes && !G.codesAvailable) return LCS_ERR_UNSUPPORTED;
    if ((implicitCodes != 0) != G.useCodes) dropGraph();
    G.useCodes = implicitCodes != 0;
    return 0;
}

LCS_API int GBT_BatchElementTables() { return G.ready && G.useCodes ? 1 : 0; }

LCS_API int GBT_BatchSetLaunch(int mode, int threads) {
    if (!G.ready || mode < 0 || mode > 2) return XPBD_ERR_BAD_ARG;
    if (mode < 2 && threads != 256 && threads != 512) return XPBD_ERR_BAD_ARG;
    if (mode == 2 && threads != 2 && threads != 4 && threads != 8) return XPBD_ERR_BAD_ARG;   // CTAs per cluster
    int rc = mode == 2 ? packClusters(threads) : packInstances(G.smCount * (threads == 512 ? 1 : 2));
    if (rc) return rc;
    G.mode = mode; G.threads = threads;
    dropGraph();
    return 0;
}

// Try every launch shape for `trialSteps` frames from the current state, keep the fastest, and put
// the state back (all shapes give bit-identical results, so the trial frames leave no trace).
// Out: mode, threads, and the ms per frame of each candidate (kAutotuneShapes floats; a shape the
// batch cannot use, e.g. a cluster too small for its largest instance, reports -1).
// Instance packing of the modes that give an instance to one CTA or cluster (0, 1, 2 as in
// packInstances); takes effect at once for the current launch shape.
LCS_API int GBT_BatchSetPacking(int packing) {
    if (!G.ready || packing < 0 || packing > 2) return XPBD_ERR_BAD_ARG;
    G.packing = packing;
    return G.mode == 0 ? 0 : GBT_BatchSetLaunch(G.mode, G.threads);
}
LCS_API int GBT_BatchPacking() { return G.ready ? G.packing : -1; }

// Try every launch configuration for `trialSteps` frames from the current state, keep the fastest, and
// put the state back (all configurations give bit-identical results, so the trial frames leave no
// trace).  Searched: the lockstep grid on either element-table form; one CTA per instance at 256 and
// 512 threads and clusters of 2, 4 and 8 CTAs, each with the three instance packings.  (A colour
// sweep closes with one synchronisation per colour in every shape: a colour reads what the
// previous one wrote.)  msOut6 gets the best time of each of the six launch shapes {0/256, 1/256,
// 1/512, 2/2, 2/4, 2/8}, -1 where a shape cannot run; GBT_BatchAutotuneTable returns every trial.
LCS_API int GBT_BatchAutotune(float dt, int trialSteps, int* modeOut, int* threadsOut, float* msOut6) {
    if (!G.ready || trialSteps <= 0) return XPBD_ERR_BAD_ARG;
    Buf<float4> savePos, savePrev, saveVel;
    CK(savePos.alloc(G.N)); CK(savePrev.alloc(G.N)); CK(saveVel.alloc(G.N));
    CK(cudaMemcpyAsync(savePos.p, G.pos.p, G.N * sizeof(float4), cudaMemcpyDeviceToDevice, G.stream));
    CK(cudaMemcpyAsync(savePrev.p, G.prev.p, G.N * sizeof(float4), cudaMemcpyDeviceToDevice, G.stream));
    CK(cudaMemcpyAsync(saveVel.p, G.vel.p, G.N * sizeof(float4), cudaMemcpyDeviceToDevice, G.stream));
    std::vector<ToolPose> keepFrom = G.toolFrom, keepTool = G.tool;
    const int shapes[6][2] = {{0, 256}, {1, 256}, {1, 512}, {2, 2}, {2, 4}, {2, 8}};
    std::vector<Batch::Trial> plan;
    for (int k = 0; k < 6; k++) {
        if (shapes[k][0] == 0) {
            if (G.codesAvailable) plan.push_back({0, 256, 0, 1, -1.f});
            plan.push_back({0, 256, 0, 0, -1.f});
        } else {
            for (int pk = 0; pk < 3; pk++) plan.push_back({shapes[k][0], shapes[k][1], pk, G.useCodes ? 1 : 0, -1.f});
        }
    }
    const bool keepCodes = G.useCodes;
    float best = 1e30f; int bestK = -1;
    if (msOut6) for (int k = 0; k < 6; k++) msOut6[k] = -1.f;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a)); CK(cudaEventCreate(&b));
    for (size_t k = 0; k < plan.size(); k++) {
        Batch::Trial& t = plan[k];
        int rc = GBT_BatchSetElementTables(t.tables);
        if (rc) return rc;
        G.packing = t.packing;
        rc = GBT_BatchSetLaunch(t.mode, t.threads);
        if (rc == LCS_ERR_UNSUPPORTED) continue;
        if (rc) return rc;
        rc = stepFrames(dt, 1, nullptr, false);   // warm-up
        if (rc) return rc;
        CK(cudaEventRecord(a, G.stream));
        for (int s = 0; s < trialSteps; s++) { rc = stepFrames(dt, 1, nullptr, false); if (rc) return rc; }
        CK(cudaEventRecord(b, G.stream));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        t.ms = ms / trialSteps;
        for (int q = 0; q < 6 && msOut6; q++)
            if (shapes[q][0] == t.mode && shapes[q][1] == t.threads && (msOut6[q] < 0.f || t.ms < msOut6[q])) msOut6[q] = t.ms;
        if (t.ms < best) { best = t.ms; bestK = (int)k; }
        CK(cudaMemcpyAsync(G.pos.p, savePos.p, G.N * sizeof(float4), cudaMemcpyDeviceToDevice, G.stream));
        CK(cudaMemcpyAsync(G.prev.p, savePrev.p, G.N * sizeof(float4), cudaMemcpyDeviceToDevice, G.stream));
        CK(cudaMemcpyAsync(G.vel.p, saveVel.p, G.N * sizeof(float4), cudaMemcpyDeviceToDevice, G.stream));
        G.toolFrom = keepFrom; G.tool = keepTool;
    }
    cudaEventDestroy(a); cudaEventDestroy(b);
    savePos.release(); savePrev.release(); saveVel.release();
    G.trials = plan;
    if (bestK < 0) { GBT_BatchSetElementTables(keepCodes ? 1 : 0); return LCS_ERR_UNSUPPORTED; }
    const Batch::Trial& w = plan[bestK];
    int rc = GBT_BatchSetElementTables(w.tables);
    if (rc) return rc;
    G.packing = w.packing;
    rc = GBT_BatchSetLaunch(w.mode, w.threads);
    if (rc) return rc;
    if (modeOut) *modeOut = w.mode;
    if (threadsOut) *threadsOut = w.threads;
    CK(cudaStreamSynchronize(G.stream));
    return 0;
}

// The last autotune's trials: up to `capacity` rows of (mode, threads, packing, element tables) in
// shape4 and their ms per frame (-1: the configuration cannot run this batch); returns the number of
// trials.
LCS_API int GBT_BatchAutotuneTable(int capacity, int* shape4, float* ms) {
    if (!G.ready || capacity < 0 || (capacity > 0 && (!shape4 || !ms))) return XPBD_ERR_BAD_ARG;
    const int n = (int)G.trials.size();
    for (int k = 0; k < n && k < capacity; k++) {
        const Batch::Trial& t = G.trials[k];
        shape4[4 * k] = t.mode; shape4[4 * k + 1] = t.threads; shape4[4 * k + 2] = t.packing; shape4[4 * k + 3] = t.tables;
        ms[k] = t.ms;
    }
    return n;
}

LCS_API void GBT_BatchProfileEnable(int enabled) {
    for (cudaEvent_t e : G.events) cudaEventDestroy(e);
    G.events.clear();
    G.profile = enabled != 0;
}
LCS_API int GBT_BatchProfileRead(float* msTotal) {
    if (!msTotal || G.events.empty()) return XPBD_ERR_BAD_ARG;
    float total = 0.f;
    for (size_t k = 0; k + 1 < G.events.size(); k += 2) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, G.events[k], G.events[k + 1]));
        total += t;
    }
    *msTotal = total;
    return 0;
}

// Debug builds (GBT_DEBUG_BOUNDS): the batch's out-of-range gather record, then cleared (release
// builds: LCS_ERR_UNSUPPORTED).
LCS_API int GBT_BatchDebugBoundsRead(unsigned* out3) {
#ifdef GBT_DEBUG_BOUNDS
    if (!G.ready || !out3 || !G.bounds.p) return XPBD_ERR_BAD_ARG;
    CK(cudaMemcpyAsync(out3, G.bounds.p, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, G.stream));
    CK(cudaMemsetAsync(G.bounds.p, 0, 3 * sizeof(unsigned), G.stream));
    CK(cudaStreamSynchronize(G.stream));
    return 0;
#else
    (void)out3;
    return LCS_ERR_UNSUPPORTED;
#endif
}

LCS_API void GBT_BatchShutdown() {
    if (G.stream) cudaStreamSynchronize(G.stream);
    releaseAll();
}
