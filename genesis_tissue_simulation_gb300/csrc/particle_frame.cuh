// Particle coordinate frames, k_ComputeParticleRot (V/physics.cu:98-205).
//
// Every live, unpinned node gets a rotation R whose column k is the world direction of its local
// lattice axis k:
//   1. axis k from the current lattice: the through-node edge (+k neighbour minus -k neighbour),
//      one-sided when only one of the two neighbours is live, skipped when neither is;
//   2. blended with the mean of the live neighbours' previous column k (kept only when the blend
//      does not nearly cancel);
//   3. a single missing axis recovered as the cross product of the other two;
//   4. R = polar factor of [axis0 axis1 axis2] by 16 Higham iterations R <- (R + R^-T) / 2;
//   identity for pinned or inactive nodes, two or more missing axes, det <= 1e-4, or an iterate that
//   has not reached orthonormality (1e-3).
//
// Records are 9 floats per node, the rows of R (RotGpu, V/cut.cuh:67).  The previous frames are a
// second buffer; the two alternate, so the "snapshot the current frames" copy of
// physics_compute_rotations (V/physics.cu:399-411) is a pointer swap.
#pragma once
#include "tissue_device.cuh"

namespace gbt {

struct Rows3 { f3 r0, r1, r2; };

GBT_HD f3 divide(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }

// det by the first row's cofactors, in the reference's operation order
GBT_HD float det3(const Rows3& m) {
    return m.r0.x * (m.r1.y * m.r2.z - m.r1.z * m.r2.y)
         - m.r0.y * (m.r1.x * m.r2.z - m.r1.z * m.r2.x)
         + m.r0.z * (m.r1.x * m.r2.y - m.r1.y * m.r2.x);
}

// R^-T = cofactor matrix / det, each cofactor formed as the adjugate entry it transposes
GBT_HD Rows3 inverseTranspose(const Rows3& m) {
    const float s = 1.0f / det3(m);
    Rows3 t;
    t.r0 = mk((m.r1.y * m.r2.z - m.r1.z * m.r2.y) * s, -(m.r1.x * m.r2.z - m.r1.z * m.r2.x) * s, (m.r1.x * m.r2.y - m.r1.y * m.r2.x) * s);
    t.r1 = mk(-(m.r0.y * m.r2.z - m.r0.z * m.r2.y) * s, (m.r0.x * m.r2.z - m.r0.z * m.r2.x) * s, -(m.r0.x * m.r2.y - m.r0.y * m.r2.x) * s);
    t.r2 = mk((m.r0.y * m.r1.z - m.r0.z * m.r1.y) * s, -(m.r0.x * m.r1.z - m.r0.z * m.r1.x) * s, (m.r0.x * m.r1.y - m.r0.y * m.r1.x) * s);
    return t;
}

__device__ __forceinline__ void storeRows(float* out, const Rows3& R) {
    out[0] = R.r0.x; out[1] = R.r0.y; out[2] = R.r0.z;
    out[3] = R.r1.x; out[4] = R.r1.y; out[5] = R.r1.z;
    out[6] = R.r2.x; out[7] = R.r2.y; out[8] = R.r2.z;
}

// Frame of node c from the node positions (xyz of pos), the live lattice `nbr` and the previous
// frames `prevRot`; writes 9 floats to `rot + 9c`.  Kept out of line, with plain pointer arguments,
// so the frame kernels that call it keep their register allocation.
static __device__ __noinline__ void particleFrame(int c, const float4* pos, const int* nbr, const int* active, const int* pinned,
                                           const float* prevRot, float* rot) {
    auto posAt = [pos](int i) { return xyz(pos[i]); };
    Rows3 R;
    R.r0 = mk(1.f, 0.f, 0.f); R.r1 = mk(0.f, 1.f, 0.f); R.r2 = mk(0.f, 0.f, 1.f);
    float* out = rot + 9 * (size_t)c;
    if (pinned[c] != 0 || active[c] == 0) { storeRows(out, R); return; }
    int nb[6];
#pragma unroll
    for (int s = 0; s < 6; s++) { int n = nbr[6 * c + s]; nb[s] = (n >= 0 && active[n] != 0) ? n : -1; }
    // mean previous column of the live neighbours, slot order 0..5, one sum per axis
    f3 psum[3] = {mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f)};
    int pc = 0;
#pragma unroll
    for (int s = 0; s < 6; s++) {
        if (nb[s] < 0) continue;
        const float* q = prevRot + 9 * (size_t)nb[s];
        psum[0] = psum[0] + mk(q[0], q[3], q[6]);
        psum[1] = psum[1] + mk(q[1], q[4], q[7]);
        psum[2] = psum[2] + mk(q[2], q[5], q[8]);
        pc++;
    }
    const f3 x = posAt(c);
    f3 axis[3];
    bool have[3] = {false, false, false};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int np = nb[2 * k + 1], nm = nb[2 * k];
        f3 e;
        if (np >= 0 && nm >= 0) e = posAt(np) - posAt(nm);
        else if (np >= 0) e = posAt(np) - x;
        else if (nm >= 0) e = x - posAt(nm);
        else continue;
        const float l = len(e);
        if (l < 1e-12f) continue;
        f3 dir = divide(e, l);
        if (pc > 0) {
            const float pl = len(psum[k]);
            if (pl > 1e-6f) {
                const f3 b = dir + divide(psum[k], pl);
                const float bl = len(b);
                if (bl > 0.25f) dir = divide(b, bl);
            }
        }
        axis[k] = dir;
        have[k] = true;
    }
    const int missing = (have[0] ? 0 : 1) + (have[1] ? 0 : 1) + (have[2] ? 0 : 1);
    if (missing == 1) {   // axis m from axis m+1 x axis m+2 (indices mod 3)
        const int miss = !have[0] ? 0 : (!have[1] ? 1 : 2);
        const f3 cx = miss == 0 ? cross(axis[1], axis[2]) : (miss == 1 ? cross(axis[2], axis[0]) : cross(axis[0], axis[1]));
        const float l = len(cx);
        if (l > 1e-9f) {
            const f3 d = divide(cx, l);
            if (miss == 0) axis[0] = d; else if (miss == 1) axis[1] = d; else axis[2] = d;
            have[0] = have[1] = have[2] = true;   // the one missing axis is recovered
        }
    }
    if (!(have[0] && have[1] && have[2])) { storeRows(out, R); return; }
    Rows3 M;
    M.r0 = mk(axis[0].x, axis[1].x, axis[2].x);
    M.r1 = mk(axis[0].y, axis[1].y, axis[2].y);
    M.r2 = mk(axis[0].z, axis[1].z, axis[2].z);
    if (det3(M) <= 1e-4f) { storeRows(out, R); return; }
    Rows3 P = M;
    for (int it = 0; it < 16; it++) {
        const Rows3 T = inverseTranspose(P);
        P.r0 = (P.r0 + T.r0) * 0.5f;
        P.r1 = (P.r1 + T.r1) * 0.5f;
        P.r2 = (P.r2 + T.r2) * 0.5f;
    }
    const f3 c0 = mk(P.r0.x, P.r1.x, P.r2.x), c1 = mk(P.r0.y, P.r1.y, P.r2.y), c2 = mk(P.r0.z, P.r1.z, P.r2.z);
    float ortho = fmaxf(fmaxf(fabsf(dot(c0, c0) - 1.f), fabsf(dot(c1, c1) - 1.f)), fabsf(dot(c2, c2) - 1.f));
    ortho = fmaxf(ortho, fmaxf(fabsf(dot(c0, c1)), fmaxf(fabsf(dot(c0, c2)), fabsf(dot(c1, c2)))));
    if (ortho > 1e-3f) { storeRows(out, R); return; }
    storeRows(out, P);
}

}  // namespace gbt
