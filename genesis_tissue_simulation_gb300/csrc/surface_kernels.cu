// Dual-contouring surface rebuild (V/dc_recon.cu:97-455 kernels, 469-487 intact advection, 507-541
// pipeline order), as one cooperative launch with grid barriers between its phases:
//   1. feature point of every surface voxel: crossings on the deformed lattice (a severed crossing is
//      rebuilt from its inside particle's frame), then either the advected rest feature point
//      (intact voxels once the rest surface exists) or the QEF gradient walk clamped to the voxel
//      box; the voxel's normal accumulator is cleared;
//      with cut voxels present, one feature point per (voxel, corner component) from its crossings
//      and cut points (the cut feature-point chain, V/cut.cu:761-985);
//   2. stitch: every surface edge's four voxels form a quad, two triangles, degenerate ones dropped,
//      then the cut walls of the cut edges.  The CTAs own contiguous edge and voxel ranges and write
//      at the prefix sums of the ranges before them, so the triangle list is in surface-edge order,
//      then voxel order, on every run (the reference appends with an atomic counter, in arrival
//      order).  With walls present, triangles over the same vertex set cancel (a hash table of
//      sorted keys, then a second prefix-sum compaction in list order).  Each kept triangle scatters
//      its area-weighted face normal to its vertices as 2^20 fixed point (integer sums: the same
//      result in any order);
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

constexpr unsigned kCutTag = 0x80000000u, kWallTag = 0x40000000u, kIdMask = 0x3FFFFFFFu;
constexpr float kPosScale = 16384.0f;        // POS_SCALE (V/cut.cuh): cut-normal sums

// Position of a triangle vertex tag (FetchPos, V/dc_recon.cu:228-234).
__device__ __forceinline__ f3 tagPos(const SurfaceMesh& s, int tag) {
    const unsigned u = (unsigned)tag;
    return (u & kCutTag) ? xyz(s.cutFP[u & kIdMask]) : xyz(s.fp[u & kIdMask]);
}

__constant__ int kStencil[3][4][3] = {{{0, 0, 0}, {0, -1, 0}, {0, -1, -1}, {0, 0, -1}},
                                      {{0, 0, 0}, {0, 0, -1}, {-1, 0, -1}, {-1, 0, 0}},
                                      {{0, 0, 0}, {-1, 0, 0}, {-1, -1, 0}, {0, -1, 0}}};
__constant__ int kStencilEdge[3][4] = {{0, 2, 6, 4}, {3, 7, 5, 1}, {8, 9, 10, 11}};
__constant__ int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ int kEdgeCorners[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

__device__ __forceinline__ bool voxIn(const SurfaceMesh& s, int x, int y, int z) {
    return x >= 0 && y >= 0 && z >= 0 && x < s.dx && y < s.dy && z < s.dz;
}
__device__ __forceinline__ int voxId(const SurfaceMesh& s, int x, int y, int z) { return x + s.dx * (y + s.dy * z); }
__device__ __forceinline__ int nodeOf(const SurfaceMesh& s, int x, int y, int z) { return x + (s.dx + 1) * (y + (s.dy + 1) * z); }
// local corner (0..7) of a voxel at offset (dx, dy, dz) from its low corner, -1 if not a corner
__device__ __forceinline__ int localCorner(int dx, int dy, int dz) {
    if ((unsigned)dx > 1u || (unsigned)dy > 1u || (unsigned)dz > 1u) return -1;
    const int b = dx | (dy << 1) | (dz << 2);
    return b == 2 ? 3 : (b == 3 ? 2 : (b == 6 ? 7 : (b == 7 ? 6 : b)));
}
__device__ __forceinline__ int compOf(const SurfaceMesh& s, unsigned mask, int lc) { return s.conn[9 * mask + 1 + lc]; }

__device__ __forceinline__ bool cutHitsMaterial(float t, float skin, int ia, int ib) {
    if (ia && ib) return true;
    if (!ia && !ib) return false;
    if (!(skin >= 0.f && skin <= 1.f)) return false;
    return ia ? t <= skin : t >= skin;
}

// Feature points of the components of cut voxel v (k_ClearCutFP, k_AccumulateCutFP,
// k_ComputeComponentFP: V/cut.cu:761-771, 791-850, 852-985).  Each component's point is seeded by
// the mean of its own crossings (the skin crossings whose owner corner lies in it) and its cut
// points, walked along the crossings' QEF gradient inside the component's deformed box, clamped to
// that box, and projected onto the plane of its cut points.  The cut points of v are those of its
// 12 edges, gathered here in a fixed order (edge, then the low owner before the high one), so the
// sums do not depend on scheduling (the reference adds them with float atomics).
// The 32 lanes of a warp work on one cut voxel (all lanes call with the same v): lane j < 24 gathers
// half-edge j's cut point (edge j / 2, low owner first) and lane k < 12 skin crossing k, all at
// once; every sum then runs in that fixed order through shuffles, and lane c < 8 finishes component
// c.  A few dependent round trips per voxel instead of one per half-edge.
__device__ __forceinline__ f3 shfl3(f3 a, int src) {
    return mk(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src), __shfl_sync(0xffffffffu, a.z, src));
}
__device__ void componentPointsWarp(const SurfaceMesh& s, int v, int lane) {
    const unsigned mask = s.cutMask[v] & 0xFFFu;
    const int vx = v % s.dx, vy = (v / s.dx) % s.dy, vz = v / (s.dx * s.dy);
    const int* c = s.voxelCorner + 8 * (size_t)v;
    const int compCount = s.conn[9 * mask];
    // corners: lane r < 8 holds corner r's id, deformed position and component
    const int cid = lane < 8 ? c[lane] : 0;
    const f3 cpos = lane < 8 ? xyz(s.pos[cid]) : mk(0.f, 0.f, 0.f);
    const int ccomp = lane < 8 ? compOf(s, mask, lane) : -1;
    // half-edge j = lane
    const int le = lane < 24 ? lane >> 1 : 0, h = lane & 1;
    const int ca = kEdgeCorners[le][0], cb = kEdgeCorners[le][1];
    const int axis = kCorner[ca][0] != kCorner[cb][0] ? 0 : (kCorner[ca][1] != kCorner[cb][1] ? 1 : 2);
    const bool aLow = kCorner[ca][axis] < kCorner[cb][axis];
    const int lcOwn = h == 0 ? (aLow ? ca : cb) : (aLow ? cb : ca);
    const int owner = __shfl_sync(0xffffffffu, cid, lcOwn);
    const int comp = __shfl_sync(0xffffffffu, ccomp, lcOwn);
    int root = 8;
    for (int q = 7; q >= 0; q--) if (__shfl_sync(0xffffffffu, ccomp, q) == comp) root = q;
    const f3 origin = shfl3(cpos, root < 8 ? root : 0);
    bool valid = false;
    f3 local = mk(0.f, 0.f, 0.f);
    int fx = 0, fy = 0, fz = 0;
    if (lane < 24) {
        const size_t slot = 6 * (size_t)owner + 2 * axis + (h == 0 ? 1 : 0);
        const float4 L = s.cutRec[2 * slot];
        if (L.w != 0.f && s.active[owner] != 0) {
            valid = true;
            const float4 Mn = s.cutRec[2 * slot + 1];
            const float* q = s.rot + 9 * (size_t)owner;
            const f3 r0 = mk(q[0], q[1], q[2]), r1 = mk(q[3], q[4], q[5]), r2 = mk(q[6], q[7], q[8]);
            const f3 lo = mk(L.x, L.y, L.z), mn = mk(Mn.x, Mn.y, Mn.z);
            local = (xyz(s.pos[owner]) - origin) + mk(dot(r0, lo), dot(r1, lo), dot(r2, lo));
            const f3 nw = mk(dot(r0, mn), dot(r1, mn), dot(r2, mn));
            fx = (int)rintf(nw.x * kPosScale); fy = (int)rintf(nw.y * kPosScale); fz = (int)rintf(nw.z * kPosScale);
        }
    }
    // lane `lane` (< 8) accumulates component `lane` in half-edge order
    f3 acc = mk(0.f, 0.f, 0.f);
    int cnt = 0, nx = 0, ny = 0, nz = 0;
    for (int j = 0; j < 24; j++) {
        const bool vj = __shfl_sync(0xffffffffu, valid, j);
        const int cj = __shfl_sync(0xffffffffu, comp, j);
        const f3 lj = shfl3(local, j);
        const int xj = __shfl_sync(0xffffffffu, fx, j), yj = __shfl_sync(0xffffffffu, fy, j), zj = __shfl_sync(0xffffffffu, fz, j);
        if (vj && cj == lane) { acc = acc + lj; cnt++; nx += xj; ny += yj; nz += zj; }
    }
    // skin crossings: lane k < ncross
    const int off = s.isectOff[v], ncross = min(s.isectCnt[v], 12);
    f3 wk = mk(0.f, 0.f, 0.f), nk = mk(0.f, 0.f, 0.f);
    int ok = -1;
    if (lane < ncross) {
        const IsectRec& it = s.isect[off + lane];
        wk = crossingWorld(s, it);
        nk = mk(it.nx, it.ny, it.nz);
        const float cT = s.cutT ? s.cutT[directedSlot(s, it.a, it.b)] : -1.f;
        const int in = skinOwnerA(it.t, cT, it.insideA) ? it.a : it.b;
        const int nxn = s.dx + 1, nyn = s.dy + 1;
        const int lc = localCorner(in % nxn - vx, (in / nxn) % nyn - vy, in / (nxn * nyn) - vz);
        ok = lc < 0 ? -1 : compOf(s, mask, lc);
    }
    f3 half = xyz(s.rest[c[6]]) - xyz(s.rest[c[0]]);
    half = mk(fabsf(half.x) * .5f, fabsf(half.y) * .5f, fabsf(half.z) * .5f);
    // component `lane`
    const int me = lane;
    f3 bc = mk(0.f, 0.f, 0.f), corigin = mk(0.f, 0.f, 0.f);
    int nCorn = 0;
    for (int q = 0; q < 8; q++) {
        const int cq = __shfl_sync(0xffffffffu, ccomp, q);
        const f3 pq = shfl3(cpos, q);
        if (cq != me) continue;
        if (nCorn == 0) corigin = pq;
        bc = bc + pq;
        nCorn++;
    }
    if (nCorn > 0) bc = mk(bc.x / (float)nCorn, bc.y / (float)nCorn, bc.z / (float)nCorn);
    f3 sum = mk(0.f, 0.f, 0.f);
    int nIncl = 0;
    for (int k = 0; k < ncross; k++) {
        const int ow = __shfl_sync(0xffffffffu, ok, k);
        const f3 w = shfl3(wk, k);
        if (ow == me) { sum = sum + w; nIncl++; }
    }
    if (cnt > 0) sum = (sum + acc) + corigin * (float)cnt;
    const int total = nIncl + cnt;
    f3 x = total > 0 ? mk(sum.x / (float)total, sum.y / (float)total, sum.z / (float)total) : mk(0.f, 0.f, 0.f);
    bool walking = nIncl > 0 && total > 0;
    for (int it = 0; it < s.qefIters; it++) {   // every lane runs every iteration (the shuffles)
        f3 F = mk(0.f, 0.f, 0.f);
        for (int k = 0; k < ncross; k++) {
            const int ow = __shfl_sync(0xffffffffu, ok, k);
            const f3 w = shfl3(wk, k), n = shfl3(nk, k);
            if (ow == me) F = F + n * dot(n, w - x);
        }
        if (walking) {
            const float a = 0.1f * (1.0f - (float)it / (float)s.qefIters);
            const f3 xn = x + F * a;
            if (fabsf(xn.x - bc.x) >= half.x || fabsf(xn.y - bc.y) >= half.y || fabsf(xn.z - bc.z) >= half.z) walking = false;
            else x = xn;
        }
    }
    if (lane >= 8) return;
    const size_t slot = 8 * (size_t)v + me;
    s.cutNrmFixed[3 * slot] = 0; s.cutNrmFixed[3 * slot + 1] = 0; s.cutNrmFixed[3 * slot + 2] = 0;
    if (me >= compCount || total == 0) { s.cutFP[slot] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    x = mk(fminf(fmaxf(x.x, bc.x - half.x), bc.x + half.x), fminf(fmaxf(x.y, bc.y - half.y), bc.y + half.y),
           fminf(fmaxf(x.z, bc.z - half.z), bc.z + half.z));
    if (cnt > 0) {
        const f3 nAcc = mk((float)nx / kPosScale, (float)ny / kPosScale, (float)nz / kPosScale);
        const float nLen = len(nAcc);
        if (nLen > 1e-6f && nLen > 0.25f * (float)cnt) {
            const f3 nbar = mk(nAcc.x / nLen, nAcc.y / nLen, nAcc.z / nLen);
            const f3 cutC = mk(acc.x / (float)cnt, acc.y / (float)cnt, acc.z / (float)cnt) + corigin;
            x = x - nbar * dot(nbar, x - cutC);
        }
    }
    s.cutFP[slot] = make_float4(x.x, x.y, x.z, 1.f);
}

// Vertex of a skin quad (StitchVertId, V/dc_recon.cu:213-226): a cut, occupied voxel resolves to
// the feature point of the component holding the crossing's inside corner, when it has one.
__device__ int stitchVert(const SurfaceMesh& s, bool cutChain, int x, int y, int z, int icx, int icy, int icz) {
    const int v = voxId(s, x, y, z);
    if (!cutChain) return v;
    const unsigned mask = s.cutMask[v] & 0xFFFu;
    if (mask == 0u || s.occupied[v] == 0u) return v;
    const int lc = localCorner(icx - x, icy - y, icz - z);
    if (lc < 0) return v;
    const int slot = 8 * v + compOf(s, mask, lc);
    return s.cutFP[slot].w > .5f ? (int)(kCutTag | (unsigned)slot) : v;
}

// The quad of surface edge e as two triangles (k_Stitch, V/dc_recon.cu:241-289): voxel stencil
// counter-clockwise about +axis, flipped when the base corner is outside; a triangle whose area
// vector is below 1e-8 is dropped.
__device__ void stitchEdge(const SurfaceMesh& s, bool cutChain, int e, int ids[6], bool ok[2]) {
    const int4 r = s.edges[e];
    const int axis = r.x & 3, insideA = r.x >> 2;
    const int ax = axis == 0, ay = axis == 1, az = axis == 2;
    int icx = r.y, icy = r.z, icz = r.w;
    if (cutChain) {   // the inside corner after a cut between it and the skin
        const int slot = 6 * nodeOf(s, r.y, r.z, r.w) + 2 * axis + 1;
        const float cT = s.cutT ? s.cutT[slot] : -1.f;
        if (!skinOwnerA(s.skinT[slot], cT, insideA)) { icx += ax; icy += ay; icz += az; }
    }
    int v[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
        v[k] = stitchVert(s, cutChain, r.y + kStencil[axis][k][0], r.z + kStencil[axis][k][1], r.w + kStencil[axis][k][2], icx, icy, icz);
    int a = v[0], b = v[1], c = v[2], d = v[3];
    if (insideA == 0) { const int t = b; b = d; d = t; }
    ids[0] = a; ids[1] = b; ids[2] = c; ids[3] = a; ids[4] = c; ids[5] = d;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const f3 p0 = tagPos(s, ids[3 * k]), p1 = tagPos(s, ids[3 * k + 1]), p2 = tagPos(s, ids[3 * k + 2]);
        const f3 n = cross(p1 - p0, p2 - p0);
        ok[k] = !(dot(n, n) < 1e-16f);
    }
}

// Wall faces of cut voxel v (k_BuildCutTriangles + EmitCutQuad, V/cut.cu:988-1089), for the cut
// edges whose first marked stencil voxel is v: from each end p of the edge, the component points
// of p's component in the four voxels around the edge, fanned (through the separated corners when
// two opposite corners are shared), wound by the rest stencil and flipped for the far end; faces
// made of shared points only, or of zero area, are dropped.  A voxel's faces come item by item,
// item j = (edge j / 2, end j % 2), in item order.  wallItem gives item j's faces: it writes them
// from out[3 * base] on (those at or beyond `cap` are skipped; none when out is null) and returns
// how many there are (at most 2).
__device__ int wallItem(const SurfaceMesh& s, int v, unsigned mask, int j, int* out, int base, int cap) {
    const int le = j >> 1, end = j & 1;
    if (((mask >> le) & 1u) == 0u) return 0;
    const int vx = v % s.dx, vy = (v / s.dx) % s.dy, vz = v / (s.dx * s.dy);
    const int ca = kEdgeCorners[le][0], cb = kEdgeCorners[le][1];
    const int axis = kCorner[ca][0] != kCorner[cb][0] ? 0 : (kCorner[ca][1] != kCorner[cb][1] ? 1 : 2);
    const int bx = vx + min(kCorner[ca][0], kCorner[cb][0]), by = vy + min(kCorner[ca][1], kCorner[cb][1]),
              bz = vz + min(kCorner[ca][2], kCorner[cb][2]);
    bool valid = true, canonical = true, seen = false;
    for (int st = 0; st < 4; st++) {
        const int x = bx + kStencil[axis][st][0], y = by + kStencil[axis][st][1], z = bz + kStencil[axis][st][2];
        if (!voxIn(s, x, y, z)) { valid = false; continue; }
        if (x == vx && y == vy && z == vz) seen = true;
        else if (!seen && ((s.cutMask[voxId(s, x, y, z)] >> kStencilEdge[axis][st]) & 1u)) canonical = false;
    }
    if (!valid || !canonical) return 0;
    const int ax = axis == 0, ay = axis == 1, az = axis == 2;
    const int A = nodeOf(s, bx, by, bz), B = nodeOf(s, bx + ax, by + ay, bz + az);
    const bool basedHere = end == 0;
    const int p = basedHere ? A : B, other = basedHere ? B : A;
    const int px = bx + (basedHere ? 0 : ax), py = by + (basedHere ? 0 : ay), pz = bz + (basedHere ? 0 : az);
    const int qx = bx + (basedHere ? ax : 0), qy = by + (basedHere ? ay : 0), qz = bz + (basedHere ? az : 0);
    const int slot = 6 * p + 2 * axis + (basedHere ? 1 : 0);
    if (!cutHitsMaterial(s.cutT[slot], s.skinT[slot], s.inside[p], s.inside[other])) return 0;
    int tag[4]; bool ok[4], shared[4]; int n = 0;
    for (int st = 0; st < 4; st++) {
        ok[st] = false; shared[st] = false; tag[st] = 0;
        const int x = bx + kStencil[axis][st][0], y = by + kStencil[axis][st][1], z = bz + kStencil[axis][st][2];
        const int w = voxId(s, x, y, z);
        if (s.occupied[w] == 0u) continue;
        const unsigned m2 = s.cutMask[w] & 0xFFFu;
        if (m2 == 0u) continue;
        const int lc = localCorner(px - x, py - y, pz - z);
        if (lc < 0) continue;
        const int comp = compOf(s, m2, lc);
        const int lq = localCorner(qx - x, qy - y, qz - z);
        shared[st] = lq >= 0 && comp == compOf(s, m2, lq);
        const int fs = 8 * w + comp;
        if (s.cutFP[fs].w < .5f) continue;
        tag[st] = (int)(kCutTag | kWallTag | (unsigned)fs);
        ok[st] = true;
        n++;
    }
    if (n < 3) return 0;
    int ord[4], m = 0;
    for (int st = 0; st < 4; st++) if (ok[st]) ord[m++] = st;
    if (m == 4 && shared[ord[0]] && shared[ord[2]] && !shared[ord[1]] && !shared[ord[3]]) {
        const int first = ord[0]; ord[0] = ord[1]; ord[1] = ord[2]; ord[2] = ord[3]; ord[3] = first;
    }
    f3 q[4];
    for (int k = 0; k < m; k++) q[k] = tagPos(s, tag[ord[k]]);
    int count = 0;
    for (int k = 1; k < m - 1; k++) {
        if (shared[ord[0]] && shared[ord[k]] && shared[ord[k + 1]]) continue;
        const f3 nrm = cross(q[k] - q[0], q[k + 1] - q[0]);
        if (dot(nrm, nrm) < 1e-16f) continue;
        const int t = base + count;
        if (out && t < cap) {
            out[3 * t] = tag[ord[0]];
            out[3 * t + 1] = tag[ord[basedHere ? k : k + 1]];
            out[3 * t + 2] = tag[ord[basedHere ? k + 1 : k]];
        }
        count++;
    }
    return count;
}
// A warp on cut voxel v (all lanes call with the same v): lane j < 24 takes item j; returns the
// voxel's face count (every lane), writing the faces from out[3 * base] on in item order when out
// is given.
__device__ int wallsOfVoxelWarp(const SurfaceMesh& s, int v, int lane, int* out, int base, int cap) {
    const unsigned mask = s.cutMask[v] & 0xFFFu;
    const int mine = lane < 24 ? wallItem(s, v, mask, lane, nullptr, 0, 0) : 0;
    int before = mine;   // inclusive scan over lanes
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, before, d);
        if (lane >= d) before += y;
    }
    const int total = __shfl_sync(0xffffffffu, before, 31);
    if (out && mine > 0) wallItem(s, v, mask, lane, out, base + before - mine, cap);
    return total;
}

// Triangle key for the internal-face cancellation (V/surface_cleanup.cuh): the three vertex tags
// without the wall marker, sorted; `odd` is the parity of the sorting permutation.
__device__ __forceinline__ void faceKey(const int* t, unsigned k[3], bool* odd) {
    for (int i = 0; i < 3; i++) k[i] = (unsigned)t[i] & 0xBFFFFFFFu;
    bool o = false;
    if (k[0] > k[1]) { const unsigned x = k[0]; k[0] = k[1]; k[1] = x; o = !o; }
    if (k[1] > k[2]) { const unsigned x = k[1]; k[1] = k[2]; k[2] = x; o = !o; }
    if (k[0] > k[1]) { const unsigned x = k[0]; k[0] = k[1]; k[1] = x; o = !o; }
    *odd = o;
}
__device__ __forceinline__ unsigned faceHash(const unsigned k[3], int fcap) {
    return ((k[0] * 73856093u) ^ (k[1] * 19349663u) ^ (k[2] * 83492791u)) & (unsigned)(fcap - 1);
}

// Face normal of triangle t scattered to its vertices as fixed point (k_NormalsScatter).
__device__ void scatterNormal(const SurfaceMesh& s, const int* t) {
    const f3 p0 = tagPos(s, t[0]), n = cross(tagPos(s, t[1]) - p0, tagPos(s, t[2]) - p0);
    const int fx = (int)(n.x * kNormalScale), fy = (int)(n.y * kNormalScale), fz = (int)(n.z * kNormalScale);
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const unsigned u = (unsigned)t[q];
        int* d = (u & kCutTag) ? s.cutNrmFixed + 3 * (size_t)(u & kIdMask) : s.nrmFixed + 3 * (size_t)u;
        atomicAdd(d, fx); atomicAdd(d + 1, fy); atomicAdd(d + 2, fz);
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
    const int r = g.rank(), R = g.size(), G = (int)gridDim.x, b = (int)blockIdx.x;
    const bool cutChain = s.cutActive && s.conn != nullptr;
    // 1. feature points of the surface voxels and of the components of cut voxels; normal sums cleared
    for (int j = r; j < s.nSurfVox; j += R) {
        const int v = s.surfVox[j];
        featurePoint(s, v);
        s.nrmFixed[3 * v] = 0; s.nrmFixed[3 * v + 1] = 0; s.nrmFixed[3 * v + 2] = 0;
    }
    // Cut voxels go a warp each, warp w taking the voxels v = w (mod warps), so a blade's
    // neighbouring cut voxels spread over the GPU.
    const int lane = (int)(threadIdx.x & 31u), W = R >> 5, wid = r >> 5;
    auto forCutVoxels = [&](auto&& work) {
        for (int k0 = 0; wid + k0 * W < s.nVox; k0 += 32) {
            const int v = wid + (k0 + lane) * W;
            const bool cut = v < s.nVox && (s.cutMask[v] & 0xFFFu) != 0u && s.occupied[v] != 0u;
            for (unsigned bits = __ballot_sync(0xffffffffu, cut); bits != 0u; bits &= bits - 1u)
                work(wid + (k0 + __ffs((int)bits) - 1) * W);
        }
    };
    if (cutChain) {
        forCutVoxels([&](int v) { componentPointsWarp(s, v, lane); });
        if (threadIdx.x == 0) s.blockTotal[G + b] = 0;   // wall faces of this CTA's voxel range, summed in 2.
    }
    if (!g.sync()) return;
    // 2. count: skin quads of this CTA's surface-edge range, cut walls of its voxel range
    const int ce = (s.nEdges + G - 1) / G, e0 = min(s.nEdges, b * ce), e1 = min(s.nEdges, e0 + ce);
    const int cv = cutChain ? (s.nVox + G - 1) / G : 0, v0 = min(s.nVox, b * cv), v1 = cutChain ? min(s.nVox, v0 + cv) : v0;
    int mine = 0;
    for (int e = e0 + (int)threadIdx.x; e < e1; e += blockDim.x) {
        int ids[6]; bool ok[2];
        stitchEdge(s, cutChain, e, ids, ok);
        mine += (ok[0] ? 1 : 0) + (ok[1] ? 1 : 0);
    }
    if (cutChain)   // each cut voxel's wall faces, added to the total of the CTA whose range holds it
        forCutVoxels([&](int v) {
            const int n = wallsOfVoxelWarp(s, v, lane, nullptr, 0, 0);
            if (lane == 0) {
                s.wallCount[v] = n;
                if (n > 0) atomicAdd(s.blockTotal + G + v / cv, n);
            }
        });
    const int ownSkin = blockSum(mine);
    if (threadIdx.x == 0) { s.blockTotal[b] = ownSkin; if (!cutChain) s.blockTotal[G + b] = 0; }
    if (!g.sync()) return;
    // write at the prefix: the skin in surface-edge order, then the walls in voxel order
    int skinBefore = 0, skinAll = 0, wallBefore = 0, wallAll = 0;
    for (int k = threadIdx.x; k < G; k += blockDim.x) {
        const int a = *(volatile int*)(s.blockTotal + k), w = *(volatile int*)(s.blockTotal + G + k);
        skinAll += a; wallAll += w;
        if (k < b) { skinBefore += a; wallBefore += w; }
    }
    skinBefore = blockSum(skinBefore); skinAll = blockSum(skinAll); wallBefore = blockSum(wallBefore); wallAll = blockSum(wallAll);
    const int T = min(skinAll + wallAll, s.triCapacity);
    const bool cancel = wallAll > 0;   // faces can only repeat where walls meet the skin or each other
    int* out = cancel ? s.raw : s.tri;
    if (!cancel && b == G - 1 && threadIdx.x == 0) *s.triCount = 3u * (unsigned)T;
    int running = skinBefore;
    for (int base = e0; base < e1; base += blockDim.x) {
        const int e = base + (int)threadIdx.x;
        int ids[6] = {0, 0, 0, 0, 0, 0};
        bool ok[2] = {false, false};
        if (e < e1) stitchEdge(s, cutChain, e, ids, ok);
        int roundTotal = 0;
        int t = running + blockExclusive((ok[0] ? 1 : 0) + (ok[1] ? 1 : 0), &roundTotal);
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if (!ok[k]) continue;
            if (t < s.triCapacity) {
                out[3 * t] = ids[3 * k]; out[3 * t + 1] = ids[3 * k + 1]; out[3 * t + 2] = ids[3 * k + 2];
                if (!cancel) scatterNormal(s, ids + 3 * k);
            }
            t++;
        }
        running += roundTotal;
    }
    running = skinAll + wallBefore;   // the walls' first faces, in voxel order
    for (int base = v0; base < v1; base += blockDim.x) {
        const int v = base + (int)threadIdx.x;
        const bool cut = v < v1 && (s.cutMask[v] & 0xFFFu) != 0u && s.occupied[v] != 0u;
        const int c = cut ? s.wallCount[v] : 0;
        int roundTotal = 0;
        const int t = running + blockExclusive(c, &roundTotal);
        if (cut) s.wallCount[v] = c > 0 ? t : -1;
        running += roundTotal;
    }
    if (!g.sync()) return;
    if (cancel) {
        // the walls at their places, a warp per cut voxel that has any
        forCutVoxels([&](int v) {
            const int first = s.wallCount[v];
            if (first >= 0) wallsOfVoxelWarp(s, v, lane, out, first, s.triCapacity);
        });
        if (!g.sync()) return;
        // internal faces (V/surface_cleanup.cuh): triangles with the same vertex set cancel in
        // opposite orientation; of a surplus the first in list order stays.  Survivors keep list order.
        int fcap = 1;
        while (fcap < 2 * T) fcap <<= 1;
        for (int k = r; k < fcap; k += R) s.faces[k] = make_int4(-1, 0, 0x7fffffff, 0x7fffffff);
        if (!g.sync()) return;
        // A triangle whose three vertices are all intact feature points (no cut tag) is never repeated:
        // its three voxels lie around exactly one surface edge, and its key differs from every key
        // holding a cut point.  Only triangles with a cut point enter the table; the others stay.
        auto intact = [&](int i) {
            return (((unsigned)s.raw[3 * i] | (unsigned)s.raw[3 * i + 1] | (unsigned)s.raw[3 * i + 2]) & kCutTag) == 0u;
        };
        for (int i = r; i < T; i += R) {
            if (intact(i)) continue;
            unsigned key[3]; bool odd;
            faceKey(s.raw + 3 * i, key, &odd);
            const unsigned h = faceHash(key, fcap);
            for (int k = 0; k < fcap; k++) {
                int4* entry = s.faces + ((h + (unsigned)k) & (unsigned)(fcap - 1));
                const int old = atomicCAS(&entry->x, -1, i);
                bool same = old < 0;
                if (!same) { unsigned o[3]; bool oo; faceKey(s.raw + 3 * old, o, &oo); same = o[0] == key[0] && o[1] == key[1] && o[2] == key[2]; }
                if (same) { atomicAdd(&entry->y, odd ? -1 : 1); atomicMin(odd ? &entry->w : &entry->z, i); break; }
            }
        }
        if (!g.sync()) return;
        const int ct = (T + G - 1) / G, t0 = min(T, b * ct), t1 = min(T, t0 + ct);
        auto keep = [&](int i) {
            if (intact(i)) return true;
            unsigned key[3]; bool odd;
            faceKey(s.raw + 3 * i, key, &odd);
            const unsigned h = faceHash(key, fcap);
            for (int k = 0; k < fcap; k++) {
                const int4 e = s.faces[(h + (unsigned)k) & (unsigned)(fcap - 1)];   // the barrier's acquire makes it current
                if (e.x < 0) return false;
                unsigned o[3]; bool oo;
                faceKey(s.raw + 3 * e.x, o, &oo);
                if (o[0] == key[0] && o[1] == key[1] && o[2] == key[2]) return e.y != 0 && i == (e.y > 0 ? e.z : e.w);
            }
            return false;
        };
        int kept = 0;
        for (int i = t0 + (int)threadIdx.x; i < t1; i += blockDim.x) kept += keep(i) ? 1 : 0;
        const int ownKept = blockSum(kept);
        if (threadIdx.x == 0) s.blockTotal[b] = ownKept;
        if (!g.sync()) return;
        int keptBefore = 0, keptAll = 0;
        for (int k = threadIdx.x; k < G; k += blockDim.x) {
            const int a = *(volatile int*)(s.blockTotal + k);
            keptAll += a;
            if (k < b) keptBefore += a;
        }
        keptBefore = blockSum(keptBefore); keptAll = blockSum(keptAll);
        if (b == G - 1 && threadIdx.x == 0) *s.triCount = 3u * (unsigned)keptAll;
        running = keptBefore;
        for (int base = t0; base < t1; base += blockDim.x) {
            const int i = base + (int)threadIdx.x;
            const bool k = i < t1 && keep(i);
            int roundTotal = 0;
            const int t = running + blockExclusive(k ? 1 : 0, &roundTotal);
            if (k) {
                s.tri[3 * t] = s.raw[3 * i]; s.tri[3 * t + 1] = s.raw[3 * i + 1]; s.tri[3 * t + 2] = s.raw[3 * i + 2];
                scatterNormal(s, s.raw + 3 * i);
            }
            running += roundTotal;
        }
        if (!g.sync()) return;
    }
    // 3. vertex soup (k_ExpandVertices V/dc_recon.cu:363-400), each vertex's unit normal formed from
    // its fixed-point sum (k_NormalsNormalize 442-455, k_NormalizeCutFP V/cut.cu:1091-1098); the rest
    // anchor of a component point is its voxel's rest skin point, else the voxel's rest centre
    const int nTri = (int)(*(volatile unsigned*)s.triCount / 3u);
    for (int i = r; i < 3 * nTri; i += R) {
        const unsigned u = (unsigned)s.tri[i];
        const int id = (int)(u & kIdMask);
        const bool cut = (u & kCutTag) != 0u;
        const float4 p = cut ? s.cutFP[id] : s.fp[id];
        const int* nf = cut ? s.cutNrmFixed + 3 * (size_t)id : s.nrmFixed + 3 * (size_t)id;
        const f3 n = mk((float)nf[0] / kNormalScale, (float)nf[1] / kNormalScale, (float)nf[2] / kNormalScale);
        const float l = len(n);
        const f3 un = l > 1e-6f ? mk(n.x / l, n.y / l, n.z / l) : mk(0.f, 0.f, 0.f);
        float4 aux;
        if (cut) {
            const int v = id >> 3;
            const float4 q = s.fpRest[v];
            const f3 anchor = q.w > 0.f ? xyz(q) : (xyz(s.rest[s.voxelCorner[8 * (size_t)v]]) + xyz(s.rest[s.voxelCorner[8 * (size_t)v + 6]])) * .5f;
            aux = make_float4(anchor.x, anchor.y, anchor.z, (float)((u >> 30) & 1u));
        } else {
            const float4 q = s.fpRest[id];
            aux = make_float4(q.x, q.y, q.z, 0.f);
        }
        s.outPos[3 * i] = p.x; s.outPos[3 * i + 1] = p.y; s.outPos[3 * i + 2] = p.z;
        s.outNrm[3 * i] = un.x; s.outNrm[3 * i + 1] = un.y; s.outNrm[3 * i + 2] = un.z;
        s.outAux[i] = aux;
    }
}

}  // namespace gbt
