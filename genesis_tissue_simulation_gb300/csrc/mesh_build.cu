// Host construction of one mesh's colour-ordered solver topology (see mesh_build.h).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "mesh_build.h"
#include "tissue_device.cuh"
#include "../../include/gbtissue.h"

namespace gbt {
namespace {

// Greedy colouring: each element takes the lowest of 64 colours none of its nodes carries yet
// (xpbd_solver.cu:1213-1230 edges, 1340-1352 bends, 1738-1751 tets).  Returns the colour count or
// XPBD_ERR_COLOR_OVERFLOW.
int colourGreedy(int count, int arity, const int* nodesOf, int nodeCount, std::vector<int>& colourOf) {
    std::vector<uint64_t> taken(nodeCount, 0);
    colourOf.resize(count);
    int colours = 0;
    for (int e = 0; e < count; e++) {
        const int* nd = nodesOf + (size_t)arity * e;
        uint64_t busy = 0;
        for (int k = 0; k < arity; k++) busy |= taken[nd[k]];
        if (busy == ~0ull) return XPBD_ERR_COLOR_OVERFLOW;
        int c = __builtin_ctzll(~busy);
        colourOf[e] = c;
        for (int k = 0; k < arity; k++) taken[nd[k]] |= 1ull << c;
        colours = std::max(colours, c + 1);
    }
    return colours;
}

// Colour-major order: offsets[c] .. offsets[c+1] hold colour c, members in element order.
void colourOrder(const std::vector<int>& colourOf, int colours, std::vector<int>& offsets, std::vector<int>& order) {
    offsets.assign(colours + 1, 0);
    for (int c : colourOf) offsets[c + 1]++;
    for (int c = 0; c < colours; c++) offsets[c + 1] += offsets[c];
    std::vector<int> fill(offsets.begin(), offsets.end() - 1);
    order.resize(colourOf.size());
    for (size_t e = 0; e < colourOf.size(); e++) order[fill[colourOf[e]]++] = (int)e;
}

bool invert3(const double a[3][3], double o[3][3], double* detOut) {
    double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1], c01 = a[1][0] * a[2][2] - a[1][2] * a[2][0], c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    double det = a[0][0] * c00 - a[0][1] * c01 + a[0][2] * c02;
    if (detOut) *detOut = det;
    if (std::fabs(det) < 1e-20) return false;
    double r = 1.0 / det;
    o[0][0] = c00 * r; o[0][1] = -(a[0][1] * a[2][2] - a[0][2] * a[2][1]) * r; o[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * r;
    o[1][0] = -c01 * r; o[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * r; o[1][2] = -(a[0][0] * a[1][2] - a[0][2] * a[1][0]) * r;
    o[2][0] = c02 * r; o[2][1] = -(a[0][0] * a[2][1] - a[0][1] * a[2][0]) * r; o[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * r;
    return true;
}

// Kuhn split of a cell along the diagonal from local corner 0 to 7; corner bit a = +axis a.
const int kKuhn[6][4] = {{0, 1, 3, 7}, {0, 3, 2, 7}, {0, 2, 6, 7}, {0, 6, 4, 7}, {0, 4, 5, 7}, {0, 5, 1, 7}};

// Tet mesh of every cell whose 8 corners are active (xpbd_build_tets, xpbd_solver.cu:1600-1848), in
// emission order (cell z, y, x; Kuhn type).
int buildTets(const MeshInput& in, float typeB[6][9], std::vector<int>& ids, std::vector<int>& owner, std::vector<int>& kind,
              std::vector<float2>& stiff) {
    auto node = [&](int x, int y, int z) { return x + (in.dx + 1) * (y + (in.dy + 1) * z); };
    const float* P = in.restPos;
    double spacing[3] = {((double)P[3 * node(in.dx, 0, 0)] - (double)P[0]) / in.dx,
                         ((double)P[3 * node(0, in.dy, 0) + 1] - (double)P[1]) / in.dy,
                         ((double)P[3 * node(0, 0, in.dz) + 2] - (double)P[2]) / in.dz};
    double typeInv[6][3][3], typeVol[6];
    for (int t = 0; t < 6; t++) {
        double Dm[3][3];
        for (int k = 1; k < 4; k++)
            for (int a = 0; a < 3; a++) Dm[a][k - 1] = ((kKuhn[t][k] >> a) & 1) * spacing[a];
        double det;
        if (!invert3(Dm, typeInv[t], &det)) return XPBD_ERR_IRREGULAR_REST;
        typeVol[t] = std::fabs(det) / 6.0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) typeB[t][3 * a + b] = (float)typeInv[t][a][b];
    }
    float mu = 1.f, kappa = 1.f;
    if (in.youngE > 0.f && in.poisson > -1.f && in.poisson < 0.5f) {
        mu = in.youngE / (2.f * (1.f + in.poisson));
        kappa = in.youngE / (3.f * (1.f - 2.f * in.poisson));
    }
    if (!(mu > 0.f)) mu = 1.f;
    if (!(kappa > 0.f)) kappa = 1.f;
    for (int z = 0; z < in.dz; z++)
        for (int y = 0; y < in.dy; y++)
            for (int x = 0; x < in.dx; x++) {
                int corner[8];
                bool full = true;
                for (int l = 0; l < 8; l++) {
                    corner[l] = node(x + (l & 1), y + ((l >> 1) & 1), z + ((l >> 2) & 1));
                    full = full && in.active[corner[l]] != 0;
                }
                if (!full) continue;
                for (int t = 0; t < 6; t++) {
                    const int* q = kKuhn[t];
                    double Dm[3][3], inv[3][3], det;
                    for (int c = 0; c < 3; c++)
                        for (int a = 0; a < 3; a++) Dm[a][c] = (double)P[3 * corner[q[c + 1]] + a] - (double)P[3 * corner[q[0]] + a];
                    if (!invert3(Dm, inv, &det)) continue;
                    if (std::fabs(det) / 6.0 < 1e-12) continue;
                    double scale = 0, dev = 0;
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) {
                            scale = std::max(scale, std::fabs(typeInv[t][a][b]));
                            dev = std::max(dev, std::fabs(inv[a][b] - typeInv[t][a][b]));
                        }
                    if (dev > 1e-4 * scale) return XPBD_ERR_IRREGULAR_REST;
                    // the three tet edges along lattice axes, owned by their lower node's +axis slot
                    int found = 0;
                    for (int a = 0; a < 4 && found < 3; a++)
                        for (int b = a + 1; b < 4 && found < 3; b++) {
                            int diff = q[a] ^ q[b];
                            if (diff != 1 && diff != 2 && diff != 4) continue;
                            int axis = diff == 1 ? 0 : (diff == 2 ? 1 : 2);
                            int low = ((q[a] >> axis) & 1) ? q[b] : q[a];
                            owner.push_back(6 * corner[low] + 2 * axis + 1);
                            found++;
                        }
                    for (int k = 0; k < 4; k++) ids.push_back(corner[q[k]]);
                    kind.push_back(t);
                    stiff.push_back(make_float2(mu * (float)typeVol[t], kappa * (float)typeVol[t]));
                }
            }
    return 0;
}

}  // namespace

int buildHostMesh(const MeshInput& in, HostMesh& out) {
    const int cc = (in.dx + 1) * (in.dy + 1) * (in.dz + 1);
    out = HostMesh();
    out.N = cc;
    // lattice edges, each from its lower node's positive slot (xpbd_bind, xpbd_solver.cu:1445-1463)
    std::vector<int> ends, owner;
    std::vector<float> restLen;
    for (int p = 0; p < cc; p++)
        for (int a = 0; a < 3; a++) {
            int slot = 6 * p + 2 * a + 1, n = in.nbrIdx[slot];
            if (n < 0) continue;
            if (n >= cc) return XPBD_ERR_BAD_ARG;
            const float* r = in.restNbr + 3 * (size_t)slot;
            ends.push_back(p); ends.push_back(n); owner.push_back(slot);
            restLen.push_back(sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]));
        }
    const int E = (int)owner.size();
    std::vector<int> colourOf, order;
    int edgeColours = colourGreedy(E, 2, ends.data(), cc, colourOf);
    if (edgeColours < 0) return edgeColours;
    colourOrder(colourOf, edgeColours, out.edgeColorOff, order);
    out.edgeEnds.resize(E); out.edgeRest.resize(E); out.edgeOwner.resize(E);
    for (int k = 0; k < E; k++) {
        int e = order[k];
        out.edgeEnds[k] = make_int2(ends[2 * e], ends[2 * e + 1]); out.edgeRest[k] = restLen[e]; out.edgeOwner[k] = owner[e];
    }
    // bend elements alive at bind time, coloured over their three nodes (xpbd_solver.cu:1465-1479)
    const BendRecord* bp = (const BendRecord*)in.bendPairs;
    std::vector<int> bNodes, bSrc; std::vector<float> bTheta;
    for (int b = 0; b < in.bendPairCount; b++) {
        if (bp[b].alive == 0) continue;
        if (bp[b].i < 0 || bp[b].i >= cc || bp[b].j < 0 || bp[b].j >= cc || bp[b].k < 0 || bp[b].k >= cc) return XPBD_ERR_BAD_ARG;
        bNodes.push_back(bp[b].i); bNodes.push_back(bp[b].j); bNodes.push_back(bp[b].k);
        bTheta.push_back(bp[b].theta0); bSrc.push_back(b);
    }
    const int B = (int)bSrc.size();
    int bendColours = colourGreedy(B, 3, bNodes.data(), cc, colourOf);
    if (bendColours < 0) return bendColours;
    colourOrder(colourOf, bendColours, out.bendColorOff, order);
    out.bendIJK.resize(B); out.bendSrc.resize(B);
    for (int k = 0; k < B; k++) {
        int e = order[k];
        float th = bTheta[e];
        int thBits; std::memcpy(&thBits, &th, 4);
        out.bendIJK[k] = make_int4(bNodes[3 * e], bNodes[3 * e + 1], bNodes[3 * e + 2], thBits);
        out.bendSrc[k] = bSrc[e];
    }
    // tets
    std::vector<int> tIds, tOwner, tKind; std::vector<float2> tStiff;
    int rc = buildTets(in, out.typeB, tIds, tOwner, tKind, tStiff);
    if (rc) return rc;
    const int T = (int)tKind.size();
    if (T % 6) return XPBD_ERR_IRREGULAR_REST;
    int tetColours = colourGreedy(T, 4, tIds.data(), cc, colourOf);
    if (tetColours < 0) return tetColours;
    colourOrder(colourOf, tetColours, out.tetColorOff, order);
    // storage index: Kuhn type major, cell order minor (xpbd_solver.cu:1757-1780)
    std::vector<int> place(T), perType(7, 0);
    for (int e = 0; e < T; e++) perType[tKind[e] + 1]++;
    for (int k = 0; k < 6; k++) perType[k + 1] += perType[k];
    for (int e = 0; e < T; e++) place[e] = perType[tKind[e]]++;
    out.tetIdsStorage.assign((size_t)4 * T, 0); out.tetStiffStorage.assign(T, make_float2(0, 0)); out.tetColorOrder.assign(T, 0);
    out.tetIds.resize(T); out.tetMeta.resize(T); out.tetOwner.resize((size_t)3 * T); out.tetStiff.resize(T);
    for (int e = 0; e < T; e++) {
        for (int k = 0; k < 4; k++) out.tetIdsStorage[4 * place[e] + k] = tIds[4 * e + k];
        out.tetStiffStorage[place[e]] = tStiff[e];
    }
    for (int k = 0; k < T; k++) {
        int e = order[k];
        out.tetColorOrder[k] = place[e];
        out.tetIds[k] = make_int4(tIds[4 * e], tIds[4 * e + 1], tIds[4 * e + 2], tIds[4 * e + 3]);
        out.tetMeta[k] = tKind[e] | 8;
        for (int o = 0; o < 3; o++) out.tetOwner[3 * k + o] = tOwner[3 * e + o];
        out.tetStiff[k] = tStiff[e];
    }
    out.E = E; out.B = B; out.T = T;
    // node state: pos.w = inverse mass, ext.w = mass
    out.pos.resize(cc); out.ext.resize(cc);
    for (int i = 0; i < cc; i++) {
        out.ext[i] = make_float4(in.extForce[3 * i], in.extForce[3 * i + 1], in.extForce[3 * i + 2], in.mass[i]);
        float w = (in.pinned[i] != 0 || in.active[i] == 0) ? 0.f : 1.f / in.mass[i];
        out.pos[i] = make_float4(in.restPos[3 * i], in.restPos[3 * i + 1], in.restPos[3 * i + 2], w);
    }
    return 0;
}

}  // namespace gbt
