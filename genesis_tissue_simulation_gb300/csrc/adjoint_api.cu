// GBT_Diff* C ABI: a differentiable rollout of the plain XPBD step on the LCS session's mesh.
//
// GBT_DiffBegin snapshots the session state as the rollout origin and sizes the checkpoint and tape
// buffers.  GBT_DiffForward runs `frames` frames from the origin with per-tet log-compliances and a
// capsule path given as device arrays (one launch), checkpointing every k substeps.
// GBT_DiffBackward takes the adjoint of the final node positions and returns the adjoints of the
// log-compliances, the capsule path, and optionally of the rest shape (per-edge rest lengths by
// slot, per-tet rest inverse matrices) and of the origin state.  All array arguments of these
// three calls are device pointers on the session's device.  The reference has no counterpart: its
// solver is not differentiable.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "adjoint_kernels.h"
#include "session_view.h"
#include "../../include/gbtissue.h"

using namespace gbt;

namespace {

template <class T> struct Dev {
    T* p = nullptr; size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

struct Diff {
    bool ready = false, haveForward = false;
    int N = 0, E = 0, T = 0, every = 5, maxFrames = 0, substeps = 1;
    float young = 0.f;
    Dev<float4> originPos, originVel, finalPos, finalVel, ckPos, ckVel, tapeQ, tapeV, tapeX, tapeEdge, tapeTet, gx, gv, gq;
    Dev<float> theta, path, gTheta, gRest, gB, pathPartial;
    Dev<float2> bake, alpha;
    Dev<int> slotStorage;
    // last forward
    int frames = 0, blocks = 1; bool grid = false, contact = false; float radius = 0.f;
    DiffCoeffs dc{};
};
Diff D;

#define CK(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) return -(int)_e; } while (0)

void releaseAll() {
    for (auto* b : {&D.originPos, &D.originVel, &D.finalPos, &D.finalVel, &D.ckPos, &D.ckVel, &D.tapeQ, &D.tapeV, &D.tapeX, &D.tapeEdge,
                    &D.tapeTet, &D.gx, &D.gv, &D.gq}) b->release();
    for (auto* b : {&D.theta, &D.path, &D.gTheta, &D.gRest, &D.gB, &D.pathPartial}) b->release();
    D.bake.release(); D.alpha.release(); D.slotStorage.release();
    D.ready = false; D.haveForward = false;
}

int blocksFor(const void* kernel, const SessionView& v) {
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kDiffThreads, 0) != cudaSuccess) return 0;
    return std::max(1, perSm) * v.smCount;
}

bool useGrid(const SessionView& v) {   // launch modes 0 (automatic) and 3 (cluster, no adjoint form): by size
    if (v.launchMode == 1) return true;
    if (v.launchMode == 2) return false;
    return !(v.T < 16384 && v.N < 32768);
}

DiffBuffers buffers() {
    DiffBuffers b{};
    b.theta = D.theta.p; b.slotStorage = D.slotStorage.p; b.bake = D.bake.p; b.young = D.young;
    b.path = D.contact ? D.path.p : nullptr; b.radius = D.radius;
    b.frames = D.frames; b.every = D.every; b.total = D.frames * D.substeps;
    b.originPos = D.originPos.p; b.originVel = D.originVel.p;
    b.ckPos = D.ckPos.p; b.ckVel = D.ckVel.p;
    b.tapeQ = D.tapeQ.p; b.tapeV = D.tapeV.p; b.tapeX = D.tapeX.p; b.tapeEdge = D.tapeEdge.p; b.tapeTet = D.tapeTet.p;
    b.gx = D.gx.p; b.gv = D.gv.p; b.gq = D.gq.p; b.gTheta = D.gTheta.p; b.gRest = D.gRest.p; b.gB = D.gB.p;
    b.pathPartial = D.pathPartial.p;
    return b;
}

// Launch one of the rollout kernels on the session stream; reads the barrier status back.
int launch(const SessionView& v, bool backward, DeviceMesh m, const DiffBuffers& b) {
    ContactParams cp = v.cp;
    DiffCoeffs dc = D.dc;
    unsigned* barrier = v.state + 1;
    CK(cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), v.stream));
    if (D.grid) {
        long long budget = (long long)((double)v.syncBudgetSeconds * 1e3 * v.clockKHz);
        DiffBuffers bb = b;
        void* args[] = {&m, &dc, &cp, &bb, &barrier, &budget};
        const void* k = backward ? (const void*)diffBackwardGrid : (const void*)diffForwardGrid;
        int blocks = blocksFor(k, v);
        if (blocks <= 0) return -(int)cudaErrorInvalidConfiguration;
        if (backward && blocks != D.blocks) return -(int)cudaErrorInvalidConfiguration;
        CK(cudaLaunchCooperativeKernel(k, dim3(blocks), dim3(kDiffThreads), args, 0, v.stream));
    } else if (backward) {
        diffBackwardBlock<<<1, kDiffThreads, 0, v.stream>>>(m, dc, cp, b);
    } else {
        diffForwardBlock<<<1, kDiffThreads, 0, v.stream>>>(m, dc, cp, b);
    }
    CK(cudaGetLastError());
    unsigned status = 0;
    CK(cudaMemcpyAsync(&status, v.state + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, v.stream));
    CK(cudaStreamSynchronize(v.stream));
    return status != 0u ? LCS_ERR_DEVICE_TIMEOUT : 0;
}

}  // namespace

LCS_API int GBT_DiffBegin(float scaleModulus, int checkpointEvery, int maxFrames) {
    releaseAll();
    SessionView v{};
    int rc = sessionView(&v);
    if (rc) return rc;
    if (!(scaleModulus > 0.f) || !std::isfinite(scaleModulus) || checkpointEvery < 1 || maxFrames < 1) return XPBD_ERR_BAD_ARG;
    // the differentiable substep: predict, lattice edges, unguarded tets, capsule contact, velocity (no guard)
    if (v.kb > 0.f || v.betaS > 0.f || v.ks <= 0.f || v.cutActive || v.contactModel != 0 || v.volumePasses > 0) return LCS_ERR_UNSUPPORTED;
    D.N = v.N; D.E = v.E; D.T = v.T; D.every = checkpointEvery; D.maxFrames = maxFrames; D.substeps = v.numSubsteps;
    D.young = scaleModulus;
    const size_t N = v.N, E = v.E, T = v.T, K = checkpointEvery;
    const size_t total = (size_t)maxFrames * v.numSubsteps, segments = (total + K - 1) / K;
    CK(D.originPos.ensure(N)); CK(D.originVel.ensure(N)); CK(D.finalPos.ensure(N)); CK(D.finalVel.ensure(N));
    CK(cudaMemcpyAsync(D.originPos.p, v.mesh.pos, N * sizeof(float4), cudaMemcpyDeviceToDevice, v.stream));
    CK(cudaMemcpyAsync(D.originVel.p, v.mesh.vel, N * sizeof(float4), cudaMemcpyDeviceToDevice, v.stream));
    CK(D.bake.ensure(T));
    if (T) CK(cudaMemcpyAsync(D.bake.p, v.mesh.tetStiff, T * sizeof(float2), cudaMemcpyDeviceToDevice, v.stream));
    CK(D.slotStorage.ensure(T));
    if (T) CK(cudaMemcpyAsync(D.slotStorage.p, v.tetColorOrder, T * sizeof(int), cudaMemcpyHostToDevice, v.stream));
    CK(D.alpha.ensure(T)); CK(D.theta.ensure(T)); CK(D.gTheta.ensure(T)); CK(D.gB.ensure(9 * T)); CK(D.gRest.ensure(E));
    CK(D.path.ensure(6 * ((size_t)maxFrames + 1)));
    CK(D.ckPos.ensure(segments * N)); CK(D.ckVel.ensure(segments * N));
    CK(D.tapeQ.ensure(K * N)); CK(D.tapeV.ensure(K * N)); CK(D.tapeX.ensure(K * N));
    CK(D.tapeEdge.ensure(2 * K * E)); CK(D.tapeTet.ensure(4 * K * T));
    CK(D.gx.ensure(N)); CK(D.gv.ensure(N)); CK(D.gq.ensure(N));
    D.grid = useGrid(v);
    D.blocks = D.grid ? blocksFor((const void*)diffBackwardGrid, v) : 1;
    if (D.blocks <= 0) return -(int)cudaErrorInvalidConfiguration;
    CK(D.pathPartial.ensure(total * D.blocks * 6));
    CK(cudaStreamSynchronize(v.stream));
    D.ready = true;
    return 0;
}

LCS_API int GBT_DiffForward(float dt, int frames, const float* logCompliance, const float* capsulePath, float capsuleRadius,
                            float* finalPos) {
    if (!D.ready) return XPBD_ERR_NOT_READY;
    SessionView v{};
    int rc = sessionView(&v);
    if (rc) return rc;
    if (v.N != D.N || v.T != D.T || v.numSubsteps != D.substeps) return XPBD_ERR_BAD_ARG;
    if (frames < 1 || frames > D.maxFrames || (D.T > 0 && !logCompliance)) return XPBD_ERR_BAD_ARG;
    if (capsulePath && !(capsuleRadius > 0.f)) return XPBD_ERR_BAD_ARG;
    const int N = D.substeps;
    float h = dt / (float)N;
    if (!(h > 0.f) || !std::isfinite(h)) return XPBD_ERR_BAD_DT;
    DiffCoeffs dc{};
    dc.h = h; dc.invH = 1.f / h; dc.invH2 = 1.f / (h * h);
    dc.alphaTilde = 1.f / (v.ks * h * h);
    dc.betaGammaHS = dc.alphaTilde * v.betaS * h;
    dc.omega = v.omega;
    dc.dampingOverH = fmaxf(0.f, v.strainDamping) / h;
    dc.velScale = (1.f - v.damping) / (1.f + v.alpha * h);
    dc.contactAlphaH2 = v.cp.contactAlpha / (h * h);
    dc.doEdges = 1;
    dc.doStrain = (D.T > 0 && v.youngE > 0.f) ? 1 : 0;
    dc.contact = capsulePath ? 1 : 0;
    D.dc = dc; D.frames = frames; D.contact = capsulePath != nullptr; D.radius = capsuleRadius;
    if (D.T) CK(cudaMemcpyAsync(D.theta.p, logCompliance, D.T * sizeof(float), cudaMemcpyDeviceToDevice, v.stream));
    if (capsulePath)
        CK(cudaMemcpyAsync(D.path.p, capsulePath, 6 * ((size_t)frames + 1) * sizeof(float), cudaMemcpyDeviceToDevice, v.stream));
    DeviceMesh m = v.mesh;
    m.tetAlpha = D.alpha.p;
    D.haveForward = false;
    rc = launch(v, false, m, buffers());
    if (rc) return rc;
    CK(cudaMemcpyAsync(D.finalPos.p, v.mesh.pos, D.N * sizeof(float4), cudaMemcpyDeviceToDevice, v.stream));
    CK(cudaMemcpyAsync(D.finalVel.p, v.mesh.vel, D.N * sizeof(float4), cudaMemcpyDeviceToDevice, v.stream));
    if (finalPos) packPositions<<<(D.N + 255) / 256, 256, 0, v.stream>>>(D.N, v.mesh.pos, finalPos);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(v.stream));
    D.haveForward = true;
    return 0;
}

LCS_API int GBT_DiffBackward(const float* gradPos, float* gradLogCompliance, float* gradCapsulePath, float* gradRestLength,
                             float* gradRestInverse, float* gradOrigin) {
    if (!D.ready || !D.haveForward) return XPBD_ERR_NOT_READY;
    if (!gradPos || (D.T > 0 && !gradLogCompliance)) return XPBD_ERR_BAD_ARG;
    SessionView v{};
    int rc = sessionView(&v);
    if (rc) return rc;
    cudaStream_t s = v.stream;
    unpackGradient<<<(D.N + 255) / 256, 256, 0, s>>>(D.N, gradPos, D.gx.p);
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(D.gv.p, 0, D.N * sizeof(float4), s));
    CK(cudaMemsetAsync(D.gq.p, 0, D.N * sizeof(float4), s));
    CK(cudaMemsetAsync(D.gTheta.p, 0, std::max(D.T, 1) * sizeof(float), s));
    const size_t total = (size_t)D.frames * D.substeps;
    if (D.contact) CK(cudaMemsetAsync(D.pathPartial.p, 0, total * D.blocks * 6 * sizeof(float), s));
    DiffBuffers b = buffers();
    if (gradRestLength) CK(cudaMemsetAsync(D.gRest.p, 0, std::max(D.E, 1) * sizeof(float), s)); else b.gRest = nullptr;
    if (gradRestInverse) CK(cudaMemsetAsync(D.gB.p, 0, 9 * (size_t)std::max(D.T, 1) * sizeof(float), s)); else b.gB = nullptr;
    DeviceMesh m = v.mesh;
    m.tetAlpha = D.alpha.p;
    rc = launch(v, true, m, b);
    if (rc) return rc;
    if (D.T) CK(cudaMemcpyAsync(gradLogCompliance, D.gTheta.p, D.T * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (gradCapsulePath) {
        int n = 6 * (D.frames + 1);
        if (D.contact) diffPathGradient<<<(n + 127) / 128, 128, 0, s>>>(b, D.blocks, D.substeps, gradCapsulePath);
        else CK(cudaMemsetAsync(gradCapsulePath, 0, n * sizeof(float), s));
    }
    if (gradRestLength) {
        CK(cudaMemsetAsync(gradRestLength, 0, (size_t)6 * D.N * sizeof(float), s));
        if (D.E) scatterSlots<<<(D.E + 255) / 256, 256, 0, s>>>(D.E, D.gRest.p, v.mesh.edgeOwner, gradRestLength);
    }
    if (gradRestInverse && D.T) scatterRows9<<<(D.T + 255) / 256, 256, 0, s>>>(D.T, D.gB.p, D.slotStorage.p, gradRestInverse);
    if (gradOrigin) {
        packPositions<<<(D.N + 255) / 256, 256, 0, s>>>(D.N, D.gx.p, gradOrigin);
        packPositions<<<(D.N + 255) / 256, 256, 0, s>>>(D.N, D.gv.p, gradOrigin + (size_t)3 * D.N);
    }
    CK(cudaGetLastError());
    // leave the session at the rollout's final state, as the forward did
    CK(cudaMemcpyAsync(v.mesh.pos, D.finalPos.p, D.N * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(v.mesh.vel, D.finalVel.p, D.N * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

LCS_API int GBT_DiffInfo(int* out4) {
    if (!D.ready || !out4) return XPBD_ERR_NOT_READY;
    out4[0] = D.grid ? 1 : 0; out4[1] = D.blocks; out4[2] = D.every; out4[3] = D.maxFrames;
    return 0;
}

LCS_API void GBT_DiffEnd() {
    SessionView v{};
    if (sessionView(&v) == 0 && v.stream) cudaStreamSynchronize(v.stream);
    releaseAll();
}
