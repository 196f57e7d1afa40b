// Cut topology of the live mesh: vertex duplication and greedy re-colouring on the device.
//
// A product of this library with no counterpart in the reference.  The reference's cut severs
// lattice links (V/cut.cu:719-746); a tet with a severed axis edge or an inactive corner stops
// being projected (k_RefreshLiveness, xpbd_solver.cu:429-466), so crossed tets are removed, and the
// colouring stays the one built at bind time (xpbd_solver.cu:1738-1780).  GBT_CutTopologyBuild
// turns the current topology into an unstructured tet mesh a consumer can take as it is:
//
//   live tets      those the liveness rule keeps, in emission order (corner-0 node ascending, then
//                  Kuhn type: the order the reference colours in), addressed by key = 6 node + type;
//   duplication    around every node its live tets are grouped by shared faces through the node
//                  (joined when they share the node and two more); groups are ranked by their first
//                  tet, the first keeps the node, group j >= 1 becomes vertex N + base(node) + j - 1
//                  with base the exclusive prefix sum of (groups - 1) in node order;
//   re-colouring   the reference's greedy first-fit colouring re-run on the live tets over the
//                  duplicated vertices: in emission order each tet takes the smallest colour that no
//                  earlier tet sharing one of its vertices holds.  This is computed in parallel as
//                  the fixed point of c(t) = mex{c(u) : u earlier than t, u shares a vertex with t},
//                  relaxed in place until a whole sweep changes nothing, starting from each tet's
//                  colour in the previous build (the bind-time colour before the first).  The
//                  recurrence has exactly one solution (induction over emission order), so the result
//                  is the sequential colouring whatever the start and the order of the sweeps; the
//                  start only decides how far changes travel, so a build after every step of cutting
//                  relaxes just that step's changes.  With nothing cut it is the bind-time colouring.
//
// The CPU restatement (oracle/cut_topology_oracle.inc) computes the same product sequentially.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/gbtissue.h"
#include "grid_sync.cuh"
#include "session_view.h"

namespace gbt {
namespace {

#define CT_CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return -(int)e_; } while (0)

constexpr int kThreads = 256;
constexpr int kMaxAround = 24;      // live tets around a lattice node: 6 + 6 (corners 0, 7) + 6 x 2
constexpr int kMaxColours = 128;    // colour masks are two 64-bit words

template <class T> struct DBuf {
    T* p = nullptr; size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        n = count;
        return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

// Buffers live from the first build until the session ends (releaseCutTopology, called by the
// session's shutdown); per-session tables are rebuilt when a new session appears.
struct CutTopologyState {
    unsigned long long generation = 0;       // session the tables below describe
    int N = 0, T = 0, keys = 0;
    DBuf<int> slotOfKey, storageOfSlot;      // key -> colour slot (-1: no tet); colour slot -> storage index
    DBuf<unsigned char> keyColour;           // each key's colour in the last build (bind-time before the first)
    DBuf<int> liveKey, rankOfKey, groupCount, dupBase, blockSums, totals;
    DBuf<unsigned char> groupOf;             // [keys][4]: group of the tet at each corner node
    DBuf<int> tetNodes, tetSource, dupParent;
    DBuf<int> nbrCount, nbrRows, upCount, upRows;   // per live tet: earlier / later neighbours, kRow-entry rows
    DBuf<unsigned char> colour, marks;
    DBuf<unsigned> sync;                     // relaxation kernel: [0] barrier counter, [1] status, [2..4] change counters, [5] sweeps, [6] overflow; [7] largest colour
    int live = 0, duplicates = 0, colours = 0, sweeps = 0;
    unsigned revision = 0;                   // topology revision of the built product
    bool built = false;
} C;

__host__ __device__ __forceinline__ int cornerPosition(int type, unsigned corner) {
    // position of Kuhn corner `corner` in the node list of a type-`type` tet (0, a, b, 7), or -1
    const unsigned a = (unsigned)(kKuhnPath >> (6 * type)) & 7u, b = (unsigned)(kKuhnPath >> (6 * type + 3)) & 7u;
    return corner == 0u ? 0 : corner == a ? 1 : corner == b ? 2 : corner == 7u ? 3 : -1;
}

// ---- session tables -------------------------------------------------------------------------
__global__ void slotTableKernel(DeviceMesh m, int T, int* slotOfKey, unsigned char* keyColour) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
        const int key = 6 * m.tetIds[k].x + (m.tetMeta[k] & 7);
        slotOfKey[key] = k;
        int c = 0;
        while (c + 1 < m.nTetColors && k >= m.tetRange[c].y) c++;
        keyColour[key] = (unsigned char)c;   // the bind-time colour
    }
}

// ---- liveness of every key (the k_RefreshLiveness rule on the current topology) ----------------
__global__ void liveKeyKernel(DeviceMesh m, int keys, const int* slotOfKey, int* liveKey) {
    for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < keys; key += gridDim.x * blockDim.x) {
        const int k = slotOfKey[key];
        int live = 0;
        if (k >= 0) {
            const int4 d = m.tetIds[k];
            const int* o = m.tetOwner + 3 * k;
            live = m.nbr[o[0]] >= 0 && m.nbr[o[1]] >= 0 && m.nbr[o[2]] >= 0 && m.active[d.x] != 0 && m.active[d.y] != 0 &&
                   m.active[d.z] != 0 && m.active[d.w] != 0;
        }
        liveKey[key] = live;
    }
}

// ---- exclusive prefix sums (three passes: block scans, a scan of the block sums, the carries) ----
__device__ __forceinline__ int blockExclusiveScan(int v, int* total) {
    __shared__ int warpSums[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) { int y = __shfl_up_sync(0xffffffffu, x, d); if (lane >= d) x += y; }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kThreads / 32 ? warpSums[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) { int y = __shfl_up_sync(0xffffffffu, w, d); if (lane >= d) w += y; }
        if (lane < kThreads / 32) warpSums[lane] = w;
    }
    __syncthreads();
    const int before = (warp > 0 ? warpSums[warp - 1] : 0) + x - v;
    if (total) *total = warpSums[kThreads / 32 - 1];
    __syncthreads();
    return before;
}
__global__ void scanBlocksKernel(const int* in, int* out, int n, int* blockSums) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    int total;
    const int v = i < n ? in[i] : 0;
    const int e = blockExclusiveScan(v, &total);
    if (i < n) out[i] = e;
    if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}
__global__ void scanSumsKernel(int* blockSums, int nb, int* grandTotal) {   // one block
    int carry = 0;
    for (int base = 0; base < nb; base += kThreads) {
        const int i = base + threadIdx.x;
        int total;
        const int v = i < nb ? blockSums[i] : 0;
        const int e = blockExclusiveScan(v, &total);
        if (i < nb) blockSums[i] = carry + e;
        carry += total;
    }
    if (threadIdx.x == 0) *grandTotal = carry;
}
__global__ void addCarryKernel(int* out, int n, const int* blockSums) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) out[i] += blockSums[blockIdx.x];
}
int exclusiveScan(const int* in, int* out, int n, int* total, cudaStream_t s) {
    const int nb = (n + kThreads - 1) / kThreads;
    CT_CK(C.blockSums.ensure(nb));
    if (n > 0) scanBlocksKernel<<<nb, kThreads, 0, s>>>(in, out, n, C.blockSums.p);
    scanSumsKernel<<<1, kThreads, 0, s>>>(C.blockSums.p, nb, total);
    if (n > 0) addCarryKernel<<<nb, kThreads, 0, s>>>(out, n, C.blockSums.p);
    CT_CK(cudaGetLastError());
    return 0;
}

// ---- the live tets around a node ------------------------------------------------------------
struct Around { int key[kMaxAround]; unsigned char corner[kMaxAround]; int count; };
// Live tets holding lattice node v, in emission (key) order, with v's position in each.
__device__ __forceinline__ void liveAround(int v, int nx, int ny, int dx, int dy, int dz, const int* liveKey, Around& a) {
    const int nxy = nx * ny;
    const int vx = v % nx, vy = (v / nx) % ny, vz = v / nxy;
    a.count = 0;
    // corner c of the cell whose corner 0 is v - offset(c); cells in decreasing c have increasing keys
    for (int c = 7; c >= 0; c--) {
        const int cx = vx - (c & 1), cy = vy - ((c >> 1) & 1), cz = vz - ((c >> 2) & 1);
        if (cx < 0 || cy < 0 || cz < 0 || cx >= dx || cy >= dy || cz >= dz) continue;
        const int u = v - cornerOffset((unsigned)c, nx, nxy);
        for (int t = 0; t < 6; t++) {
            const int pos = cornerPosition(t, (unsigned)c);
            if (pos < 0 || !liveKey[6 * u + t]) continue;
            a.key[a.count] = 6 * u + t;
            a.corner[a.count] = (unsigned char)pos;
            a.count++;
        }
    }
}

// Groups of the live tets around every node: joined through shared faces (a second and a third
// common node), ranked by their first tet in emission order.
__global__ void groupKernel(int N, int nx, int ny, int dx, int dy, int dz, const int* liveKey, unsigned char* groupOf, int* groupCount) {
    const int nxy = nx * ny;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
        Around a;
        liveAround(v, nx, ny, dx, dy, dz, liveKey, a);
        int4 nodes[kMaxAround];
        unsigned char parent[kMaxAround];
        for (int i = 0; i < a.count; i++) {
            nodes[i] = kuhnNodes(a.key[i] % 6, a.key[i] / 6, nx, nxy);
            parent[i] = (unsigned char)i;
        }
        auto find = [&](int i) { while (parent[i] != i) i = parent[i]; return i; };
        for (int i = 0; i < a.count; i++)
            for (int j = i + 1; j < a.count; j++) {
                const int4 p = nodes[i], q = nodes[j];
                const int common = (p.x == q.x) + (p.x == q.y) + (p.x == q.z) + (p.x == q.w) + (p.y == q.x) + (p.y == q.y) +
                                   (p.y == q.z) + (p.y == q.w) + (p.z == q.x) + (p.z == q.y) + (p.z == q.z) + (p.z == q.w) +
                                   (p.w == q.x) + (p.w == q.y) + (p.w == q.z) + (p.w == q.w);
                if (common < 3) continue;
                const int ri = find(i), rj = find(j);
                if (ri != rj) parent[max(ri, rj)] = (unsigned char)min(ri, rj);   // a root is its group's first member
            }
        unsigned char label[kMaxAround];
        int groups = 0;
        for (int i = 0; i < a.count; i++) {
            const int root = find(i);
            label[i] = root == i ? (unsigned char)groups++ : label[root];
            groupOf[4 * (size_t)a.key[i] + a.corner[i]] = label[i];
        }
        groupCount[v] = groups > 1 ? groups - 1 : 0;
    }
}

// ---- the live tets in emission order over the duplicated vertices -----------------------------
__device__ __forceinline__ int vertexOf(int node, int group, int N, const int* dupBase) {
    return group == 0 ? node : N + dupBase[node] + group - 1;
}
__global__ void emitKernel(int keys, int N, int nx, int nxy, const int* liveKey, const int* rankOfKey, const int* slotOfKey,
                           const int* storageOfSlot, const unsigned char* keyColour, const unsigned char* groupOf,
                           const int* dupBase, int* tetNodes, int* tetSource, unsigned char* colour) {
    for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < keys; key += gridDim.x * blockDim.x) {
        if (!liveKey[key]) continue;
        const int r = rankOfKey[key], slot = slotOfKey[key];
        const int4 d = kuhnNodes(key % 6, key / 6, nx, nxy);
        const int node[4] = {d.x, d.y, d.z, d.w};
        for (int k = 0; k < 4; k++) tetNodes[4 * (size_t)r + k] = vertexOf(node[k], groupOf[4 * (size_t)key + k], N, dupBase);
        tetSource[r] = storageOfSlot[slot];
        // the relaxation starts from the tet's colour in the previous build (the bind-time colour
        // before the first): its fixed point does not depend on the start, and after one more step
        // of cutting only the changes since that build have to travel
        colour[r] = keyColour[key];
    }
}
__global__ void keepColoursKernel(int keys, const int* liveKey, const int* rankOfKey, const unsigned char* colour,
                                  unsigned char* keyColour, unsigned* largest) {
    unsigned most = 0u;
    for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < keys; key += gridDim.x * blockDim.x)
        if (liveKey[key]) {
            const unsigned char c = colour[rankOfKey[key]];
            keyColour[key] = c;
            most = max(most, (unsigned)c);
        }
    most = __reduce_max_sync(0xffffffffu, most);
    if ((threadIdx.x & 31) == 0) atomicMax(largest, most);
}
__global__ void dupParentKernel(int N, const int* groupCount, const int* dupBase, int* dupParent) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
        for (int j = 0; j < groupCount[v]; j++) dupParent[dupBase[v] + j] = v;
}

// Neighbours of every live tet that share one of its (duplicated) vertices, in one pass: the
// earlier ones in emission order into its row of nbrRows (they decide its colour), the later ones
// into its row of upRows (they are re-evaluated when its colour changes).  A tet sharing an edge or
// a face appears once per shared vertex; the colour masks and the marks built from the rows are
// idempotent, so the rows are not deduplicated.  A row holds at most 4 x (kMaxAround - 1) entries.
// Around each corner the candidates (8 cells, the Kuhn types of each that hold the corner) are
// unrolled, their liveness, group and rank loaded together.
constexpr int kRow = 4 * kMaxAround;
__global__ void neighbourKernel(int keys, int nx, int ny, int dx, int dy, int dz, const int* liveKey, const int* rankOfKey,
                                const unsigned char* groupOf, int* nbrCount, int* nbrRows, int* upCount, int* upRows) {
    const int nxy = nx * ny;
    for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < keys; key += gridDim.x * blockDim.x) {
        if (!liveKey[key]) continue;
        const int r = rankOfKey[key];
        const int4 d = kuhnNodes(key % 6, key / 6, nx, nxy);
        const int node[4] = {d.x, d.y, d.z, d.w};
        int* down = nbrRows + (size_t)r * kRow;
        int* up = upRows + (size_t)r * kRow;
        int nd = 0, nu = 0;
        for (int k = 0; k < 4; k++) {
            const int v = node[k];
            const unsigned char g = groupOf[4 * (size_t)key + k];
            const int vx = v % nx, vy = (v / nx) % ny, vz = v / nxy;
#pragma unroll
            for (int c = 7; c >= 0; c--) {
                const int cx = vx - (c & 1), cy = vy - ((c >> 1) & 1), cz = vz - ((c >> 2) & 1);
                const bool inside = cx >= 0 && cy >= 0 && cz >= 0 && cx < dx && cy < dy && cz < dz;
                const int u = v - cornerOffset((unsigned)c, nx, nxy);
#pragma unroll
                for (int t = 0; t < 6; t++) {
                    const int pos = cornerPosition(t, (unsigned)c);
                    if (pos < 0) continue;
                    const int kk = 6 * u + t;
                    const int live = inside ? liveKey[kk] : 0;
                    const unsigned char gg = inside ? groupOf[4 * (size_t)kk + pos] : (unsigned char)0xFF;
                    const int rank = inside ? rankOfKey[kk] : 0;
                    if (!live || kk == key || gg != g) continue;
                    if (kk < key) down[nd++] = rank;
                    else up[nu++] = rank;
                }
            }
        }
        nbrCount[r] = nd;
        upCount[r] = nu;
    }
}

// In-place relaxation of c(t) = mex{c(u) : u in t's earlier neighbours} over the whole grid, one
// sweep per grid barrier, until a sweep changes nothing.  Only marked tets are evaluated: every tet
// in the first sweep, afterwards those with an earlier neighbour that changed in the previous sweep
// (a tet whose earlier neighbours kept their colours since it was evaluated still satisfies the
// recurrence; a change after its evaluation marks it again).  Marks alternate between two byte
// arrays by sweep parity.  Change counters rotate over three words: sweep s counts into word s % 3,
// every block reads it after the sweep's barrier, and block 0 clears word (s + 1) % 3 during sweep
// s (its last reader finished before the previous barrier).
// A sweep lasts as long as its slowest thread, whose evaluations are chains of dependent loads (row
// entry, then the colour it names).  Tets are dealt to threads with the grid's stride, which spreads
// the marks (clustered in emission order around the cut) over the grid; a thread reads its kBatch
// marks together and every row kBatch entries at a time, so an evaluation is a few round trips.
constexpr int kBatch = 16;
static_assert(kRow % kBatch == 0, "a batch never runs past its row");
// kBatch entries of a row from `p` (16-byte aligned: rows are kRow ints, batches start at multiples
// of kBatch), the first `valid` of them kept and the rest -1.
__device__ __forceinline__ void loadRowBatch(const int* p, int valid, int (&out)[kBatch]) {
#pragma unroll
    for (int q = 0; q < kBatch / 4; q++) {
        const int4 v = reinterpret_cast<const int4*>(p)[q];
        out[4 * q] = 4 * q < valid ? v.x : -1;
        out[4 * q + 1] = 4 * q + 1 < valid ? v.y : -1;
        out[4 * q + 2] = 4 * q + 2 < valid ? v.z : -1;
        out[4 * q + 3] = 4 * q + 3 < valid ? v.w : -1;
    }
}
__global__ void __launch_bounds__(kThreads) recolourKernel(int L, const int* nbrCount, const int* nbrRows, const int* upCount,
                                                          const int* upRows, unsigned char* colour, unsigned char* marks,
                                                          unsigned* sync, long long budget, int maxSweeps) {
    GridSync g{sync, sync + 1, gridDim.x, 0u, budget, 0u};
    const int R = gridDim.x * blockDim.x, r0 = blockIdx.x * blockDim.x + threadIdx.x;
    volatile unsigned char* col = colour;
    for (int s = 0; s < maxSweeps; s++) {
        if (blockIdx.x == 0 && threadIdx.x == 0) sync[2 + (s + 1) % 3] = 0u;
        unsigned char* cur = marks + (size_t)(s & 1) * L;
        unsigned char* next = marks + (size_t)((s + 1) & 1) * L;
        bool changed = false;
        for (long long t0 = r0; t0 < L; t0 += (long long)kBatch * R) {
            unsigned marked = 0u;
#pragma unroll
            for (int u = 0; u < kBatch; u++)
                if (t0 + (long long)u * R < L && cur[t0 + (long long)u * R]) marked |= 1u << u;
            for (; marked; marked &= marked - 1u) {
                const int t = (int)(t0 + (long long)(__ffs((int)marked) - 1) * R);
                cur[t] = 0;
                const int* nbrList = nbrRows + (size_t)t * kRow;
                const int e = nbrCount[t];
                const unsigned own = col[t];
                unsigned long long m0 = 0ull, m1 = 0ull;
                for (int j = 0; j < e; j += kBatch) {
                    int nb[kBatch];
                    loadRowBatch(nbrList + j, e - j, nb);
                    unsigned c[kBatch];
#pragma unroll
                    for (int q = 0; q < kBatch; q++) c[q] = nb[q] >= 0 ? (unsigned)col[nb[q]] : 0xFFu;
#pragma unroll
                    for (int q = 0; q < kBatch; q++) {
                        if (c[q] < 64u) m0 |= 1ull << c[q];
                        else if (c[q] < 128u) m1 |= 1ull << (c[q] - 64u);
                    }
                }
                const int mex = ~m0 ? __ffsll((long long)~m0) - 1 : (~m1 ? 64 + __ffsll((long long)~m1) - 1 : kMaxColours);
                if (mex >= kMaxColours) { atomicOr(sync + 6, 1u); continue; }
                if ((unsigned)mex == own) continue;
                col[t] = (unsigned char)mex;
                changed = true;
                const int* upList = upRows + (size_t)t * kRow;
                const int ue = upCount[t];
                for (int j = 0; j < ue; j += kBatch) {
                    int up[kBatch];
                    loadRowBatch(upList + j, ue - j, up);
#pragma unroll
                    for (int q = 0; q < kBatch; q++)
                        if (up[q] >= 0) next[up[q]] = 1;
                }
            }
        }
        if (__syncthreads_or(changed) && threadIdx.x == 0) atomicAdd(sync + 2 + s % 3, 1u);
        if (!g.sync()) return;
        const unsigned any = *(volatile unsigned*)(sync + 2 + s % 3);
        if (any == 0u || *(volatile unsigned*)(sync + 6) != 0u) {
            if (blockIdx.x == 0 && threadIdx.x == 0) sync[5] = (unsigned)(s + 1);
            return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sync[5] = (unsigned)(maxSweeps + 1);   // not settled (cannot happen: maxSweeps > L)
}

int readTotal(int* dst, cudaStream_t s) {
    CT_CK(cudaMemcpyAsync(dst, C.totals.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CT_CK(cudaStreamSynchronize(s));
    return 0;
}

int build(const SessionView& v) {
    const DeviceMesh& m = v.mesh;
    const cudaStream_t s = v.stream;
    const int N = v.N, T = v.T, keys = 6 * N;
    const int nx = m.dx + 1, ny = m.dy + 1;
    auto blocks = [&](long long n) { return (int)std::max(1LL, std::min<long long>((n + kThreads - 1) / kThreads, 16LL * v.smCount)); };
    if (C.generation != v.generation || C.N != N || C.T != T) {   // per-session tables
        C.built = false;
        CT_CK(C.slotOfKey.ensure(keys)); CT_CK(C.keyColour.ensure(keys)); CT_CK(C.storageOfSlot.ensure(T));
        CT_CK(cudaMemsetAsync(C.slotOfKey.p, 0xFF, (size_t)keys * sizeof(int), s));
        CT_CK(cudaMemcpyAsync(C.storageOfSlot.p, v.tetColorOrder, (size_t)T * sizeof(int), cudaMemcpyHostToDevice, s));
        if (T > 0) slotTableKernel<<<blocks(T), kThreads, 0, s>>>(m, T, C.slotOfKey.p, C.keyColour.p);
        CT_CK(cudaGetLastError());
        CT_CK(cudaStreamSynchronize(s));   // the host table copied above is the session's, valid now
        C.generation = v.generation; C.N = N; C.T = T; C.keys = keys;
    }
    // The product depends on the neighbour table and the active flags alone.  Within one generation
    // (a physics session, cut module or restored state) they change only by severing, which counts
    // every link it removes in the revision: with the revision unchanged the last product stands.
    unsigned revision = 0;
    if (v.revision) {
        CT_CK(cudaMemcpyAsync(&revision, v.revision, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        CT_CK(cudaStreamSynchronize(s));
    }
    if (C.built && revision == C.revision) {
        C.sweeps = 0;
        return 0;
    }
    C.built = false;   // until this build completes: a failed build leaves nothing for the getter
    CT_CK(C.liveKey.ensure(keys)); CT_CK(C.rankOfKey.ensure(keys)); CT_CK(C.groupOf.ensure((size_t)4 * keys));
    CT_CK(C.groupCount.ensure(N)); CT_CK(C.dupBase.ensure(N)); CT_CK(C.totals.ensure(1)); CT_CK(C.sync.ensure(8));
    liveKeyKernel<<<blocks(keys), kThreads, 0, s>>>(m, keys, C.slotOfKey.p, C.liveKey.p);
    CT_CK(cudaGetLastError());
    int rc = exclusiveScan(C.liveKey.p, C.rankOfKey.p, keys, C.totals.p, s);
    if (rc) return rc;
    int L = 0, D = 0;
    if ((rc = readTotal(&L, s))) return rc;
    groupKernel<<<blocks(N), kThreads, 0, s>>>(N, nx, ny, m.dx, m.dy, m.dz, C.liveKey.p, C.groupOf.p, C.groupCount.p);
    CT_CK(cudaGetLastError());
    if ((rc = exclusiveScan(C.groupCount.p, C.dupBase.p, N, C.totals.p, s))) return rc;
    if ((rc = readTotal(&D, s))) return rc;
    CT_CK(C.tetNodes.ensure((size_t)4 * L)); CT_CK(C.tetSource.ensure(L)); CT_CK(C.colour.ensure(L)); CT_CK(C.dupParent.ensure(D));
    CT_CK(C.nbrCount.ensure(L)); CT_CK(C.nbrRows.ensure((size_t)kRow * L)); CT_CK(C.upCount.ensure(L)); CT_CK(C.upRows.ensure((size_t)kRow * L));
    emitKernel<<<blocks(keys), kThreads, 0, s>>>(keys, N, nx, nx * ny, C.liveKey.p, C.rankOfKey.p, C.slotOfKey.p, C.storageOfSlot.p,
                                                  C.keyColour.p, C.groupOf.p, C.dupBase.p, C.tetNodes.p, C.tetSource.p, C.colour.p);
    dupParentKernel<<<blocks(N), kThreads, 0, s>>>(N, C.groupCount.p, C.dupBase.p, C.dupParent.p);
    neighbourKernel<<<blocks(keys), kThreads, 0, s>>>(keys, nx, ny, m.dx, m.dy, m.dz, C.liveKey.p, C.rankOfKey.p, C.groupOf.p,
                                                       C.nbrCount.p, C.nbrRows.p, C.upCount.p, C.upRows.p);
    CT_CK(cudaGetLastError());
    unsigned sweeps = 0, overflow = 0;
    int colours = 0;
    if (L > 0) {
        CT_CK(C.marks.ensure((size_t)2 * L));
        CT_CK(cudaMemsetAsync(C.marks.p, 1, (size_t)L, s));                    // the first sweep evaluates every tet
        CT_CK(cudaMemsetAsync(C.marks.p + L, 0, (size_t)L, s));
        CT_CK(cudaMemsetAsync(C.sync.p, 0, 8 * sizeof(unsigned), s));
        int perSm = 0;
        CT_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, recolourKernel, kThreads, 0));
        // two CTAs per SM: after the first sweep few tets are marked, and every CTA arrives at each barrier
        const int grid = std::max(1, std::min(std::min(perSm, 2) * v.smCount, (L + kThreads - 1) / kThreads));
        long long budget = (long long)(v.syncBudgetSeconds * 1e3 * (double)v.clockKHz);
        int Lk = L, maxSweeps = L + 1;
        const int* cnt = C.nbrCount.p; const int* rows = C.nbrRows.p; const int* ucnt = C.upCount.p; const int* urows = C.upRows.p;
        unsigned char* col = C.colour.p; unsigned char* mk = C.marks.p; unsigned* sy = C.sync.p;
        void* args[] = {&Lk, &cnt, &rows, &ucnt, &urows, &col, &mk, &sy, &budget, &maxSweeps};
        CT_CK(cudaLaunchCooperativeKernel((const void*)recolourKernel, dim3(grid), dim3(kThreads), args, 0, s));
        // the colours become the next build's start (any start relaxes to the same colouring) and
        // their largest + 1 the colour count
        keepColoursKernel<<<blocks(keys), kThreads, 0, s>>>(keys, C.liveKey.p, C.rankOfKey.p, C.colour.p, C.keyColour.p, C.sync.p + 7);
        CT_CK(cudaGetLastError());
        unsigned h[8];
        CT_CK(cudaMemcpyAsync(h, C.sync.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        CT_CK(cudaStreamSynchronize(s));
        if (h[1] != 0u) return LCS_ERR_DEVICE_TIMEOUT;
        sweeps = h[5]; overflow = h[6];
        if (overflow || sweeps > (unsigned)L + 1u) return XPBD_ERR_COLOR_OVERFLOW;
        colours = (int)h[7] + 1;
    }
    C.live = L; C.duplicates = D; C.colours = colours; C.sweeps = (int)sweeps; C.revision = revision; C.built = true;
    return 0;
}

}  // namespace

void releaseCutTopology() {
    for (auto* b : {&C.slotOfKey, &C.storageOfSlot, &C.liveKey, &C.rankOfKey, &C.groupCount, &C.dupBase, &C.blockSums, &C.totals,
                    &C.tetNodes, &C.tetSource, &C.dupParent, &C.nbrCount, &C.nbrRows, &C.upCount, &C.upRows}) b->release();
    C.keyColour.release(); C.groupOf.release(); C.colour.release(); C.marks.release(); C.sync.release();
    C.generation = 0; C.built = false; C.live = C.duplicates = C.colours = C.sweeps = 0; C.revision = 0;
}

}  // namespace gbt

using namespace gbt;

LCS_API int GBT_CutTopologyBuild(int* counts4) {
    if (!counts4) return XPBD_ERR_BAD_ARG;
    SessionView v{};
    int rc = sessionView(&v);
    if (rc) return rc;
    rc = build(v);
    if (rc) return rc;
    counts4[0] = C.live; counts4[1] = C.duplicates; counts4[2] = C.colours; counts4[3] = C.sweeps;
    return 0;
}

LCS_API int GBT_GetCutTopology(int* tetNodes4L, int* tetSourceL, int* tetColourL, int* dupParentD) {
    SessionView v{};
    int rc = sessionView(&v);
    if (rc) return rc;
    if (!C.built || C.generation != v.generation) return XPBD_ERR_NOT_READY;
    if (!tetNodes4L || !tetSourceL || !tetColourL || (C.duplicates > 0 && !dupParentD)) return XPBD_ERR_BAD_ARG;
    const size_t L = (size_t)C.live;
    std::vector<unsigned char> colour(L);
    if (L > 0) {
        CT_CK(cudaMemcpyAsync(tetNodes4L, C.tetNodes.p, 4 * L * sizeof(int), cudaMemcpyDeviceToHost, v.stream));
        CT_CK(cudaMemcpyAsync(tetSourceL, C.tetSource.p, L * sizeof(int), cudaMemcpyDeviceToHost, v.stream));
        CT_CK(cudaMemcpyAsync(colour.data(), C.colour.p, L, cudaMemcpyDeviceToHost, v.stream));
    }
    if (C.duplicates > 0)
        CT_CK(cudaMemcpyAsync(dupParentD, C.dupParent.p, (size_t)C.duplicates * sizeof(int), cudaMemcpyDeviceToHost, v.stream));
    CT_CK(cudaStreamSynchronize(v.stream));
    for (size_t t = 0; t < L; t++) tetColourL[t] = colour[t];
    return 0;
}
