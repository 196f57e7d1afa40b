// Reverse-mode (adjoint) projections of the XPBD substep, one element at a time.
//
// Each function takes what the forward projection read (the element's node positions before it
// was applied, the substep-start positions, its compliance) and the adjoint of what it wrote, and
// returns the adjoint of what it read.  The forward quantities are re-evaluated with the forward's
// own operations first, so every branch (inactive element, degenerate denominators, contact gate,
// displacement cap, clamps) is taken exactly as the forward took it; the derivative of a branch
// that left its inputs unchanged is the identity.
//
// Forward formulas (unguarded Neo-Hookean block, k_solve_tet, xpbd_solver.cu:749-829; lattice
// edges, k_solve_edges, xpbd_solver.cu:484-524; capsule contact, k_SolveCCDContact,
// xpbd_solver.cu:1049-1093) are those of tissue_device.cuh; the derivation is plain reverse-mode
// differentiation of those expressions, written out term by term.
#pragma once
#include "tissue_device.cuh"

namespace gbt {

// exp(x) for the compliance map, identical on host and device: x = k ln2 + r with |r| <= ln2/2,
// ln 2 split into an exactly representable head and a tail (Cody and Waite's argument reduction,
// "Software Manual for the Elementary Functions", 1980), exp(r) by its Taylor series to degree 7
// (truncation below 6e-9 relative), 2^k from exponent bits.  x is clamped to [-87, 88].
GBT_HD float expCW(float x) {
    x = fminf(fmaxf(x, -87.f), 88.f);
    float k = rintf(x * 1.44269504f);
    float r = (x - k * 0.693359375f) - k * -2.12194440e-4f;
    float p = 1.f / 5040.f;
    p = p * r + 1.f / 720.f;
    p = p * r + 1.f / 120.f;
    p = p * r + 1.f / 24.f;
    p = p * r + 1.f / 6.f;
    p = p * r + 0.5f;
    p = p * r + 1.f;
    p = p * r + 1.f;
#ifdef __CUDA_ARCH__
    float two = __int_as_float(((int)k + 127) << 23);
#else
    int bits = ((int)k + 127) << 23;
    float two;
    __builtin_memcpy(&two, &bits, 4);
#endif
    return p * two;
}

// Per-tet compliances over h^2 from a log-compliance: the tet's baked stiffness (mu V, kappa V) is
// scaled by 1 / (exp(theta) E0), E0 the Young's modulus the bake used; d alpha / d theta = alpha.
GBT_HD float2 tetAlphaFromLog(float theta, float young, float2 bake, float invH2) {
    float s = 1.f / (expCW(theta) * young);
    float2 a;
    a.x = invH2 / (bake.x * s);
    a.y = invH2 / (bake.y * s);
    return a;
}

// Coefficients of the differentiable substep (the subset of FrameCoeffs it supports).
struct DiffCoeffs {
    float h, invH, invH2, alphaTilde, betaGammaHS, omega, dampingOverH, velScale, contactAlphaH2;
    int doEdges, doStrain, contact;
};

// ---------------------------------------------------------------------------------------------
// lattice edge
// ---------------------------------------------------------------------------------------------
// Forward: d = pi - pj, L = |d|, n = d (1/L), C = L - L0, g = n.((pi - qi) - (pj - qj)),
// dl = (-C - gamma g) / ((1 + gamma)(wi + wj) + alpha), ap = omega dl, pi += n wi ap, pj -= n wj ap.
struct EdgeAdjoint { f3 gpi, gpj, gqi, gqj; float grest; };
__device__ __forceinline__ EdgeAdjoint edgeVJP(float4 Pi, float4 Pj, f3 qi, f3 qj, float rest, float alphaTilde, float gamma,
                                               float omega, f3 ga, f3 gb) {
    EdgeAdjoint o;
    o.gpi = ga; o.gpj = gb; o.gqi = mk(0.f, 0.f, 0.f); o.gqj = o.gqi; o.grest = 0.f;
    float wi = Pi.w, wj = Pj.w, ws = wi + wj;
    if (ws <= 0.f) return o;
    f3 pi = xyz(Pi), pj = xyz(Pj);
    f3 d = pi - pj;
    float L = sqrtf(dotF(d, d));   // the forward's operations (solveEdge), fused where it fuses
    if (L < 1e-9f) return o;
    float inv = 1.f / L;
    f3 n = d * inv;
    float C = L - rest;
    f3 u = (pi - qi) - (pj - qj);
    float gdx = dotF(n, u);
    float den = fmaf(1.f + gamma, ws, alphaTilde);
    float dl = (gamma != 0.f ? fmaf(-gamma, gdx, -C) : -C) / den;
    float ap = omega * dl;
    // a = pi + n (wi ap), b = pj - n (wj ap)
    f3 gn = ga * (wi * ap) - gb * (wj * ap);
    float gap = wi * dot(ga, n) - wj * dot(gb, n);
    float gdl = omega * gap;
    float gC = -(gdl / den);
    float ggdx = -((gamma * gdl) / den);
    o.grest = -gC;
    // g = n.u
    gn = gn + u * ggdx;
    f3 gu = n * ggdx;
    o.gpi = o.gpi + gu; o.gpj = o.gpj - gu;
    o.gqi = mk(0.f, 0.f, 0.f) - gu; o.gqj = gu;
    // n = d inv, inv = 1/L, L = |d|, C = L - L0
    float gL = gC - dot(gn, d) * (inv * inv);
    f3 gd = gn * inv + n * gL;
    o.gpi = o.gpi + gd; o.gpj = o.gpj - gd;
    return o;
}

// ---------------------------------------------------------------------------------------------
// Neo-Hookean tet
// ---------------------------------------------------------------------------------------------
struct TetAdjoint { f3 gp[4], gq[4]; float gad, gah; float gB[9]; };

// P: positions (xyz, inverse mass) before the projection; q: substep-start positions; Bm: rest
// inverse (row major); ad/ah: deviatoric/hydrostatic compliance over h^2; go: adjoint of the
// projected positions.  wantB: also return the adjoint of Bm (rest shape).
__device__ __forceinline__ void tetVJP(const float* Bm, const float4 P[4], const f3 q[4], float ad, float ah, float dampingOverH,
                                       float omega, const f3 go[4], bool wantB, TetAdjoint& out) {
    const f3 zero = mk(0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 4; c++) { out.gp[c] = go[c]; out.gq[c] = zero; }
    out.gad = 0.f; out.gah = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) out.gB[k] = 0.f;
    // ---- forward, as applyTet ----
    f3 p[4] = {xyz(P[0]), xyz(P[1]), xyz(P[2]), xyz(P[3])};
    f3 br[3] = {mk(Bm[0], Bm[1], Bm[2]), mk(Bm[3], Bm[4], Bm[5]), mk(Bm[6], Bm[7], Bm[8])};
    f3 e[3] = {p[1] - p[0], p[2] - p[0], p[3] - p[0]};
    f3 F[3];
#pragma unroll
    for (int c = 0; c < 3; c++) F[c] = fmv(e[2], comp(br[2], c), fmv(e[1], comp(br[1], c), e[0] * comp(br[0], c)));
    float I1 = dotF(F[0], F[0]) + dotF(F[1], F[1]) + dotF(F[2], F[2]);
    f3 cof[3] = {crossF(F[1], F[2]), crossF(F[2], F[0]), crossF(F[0], F[1])};
    float J = dotF(F[0], cof[0]), pJ = fmaxf(J, .05f);
    float iso = powMinusTwoThirds(pJ);
    float qv = fmaf(iso, I1, -3.f);
    float q0 = fmaxf(qv, 0.f);
    float CD = sqrtf(fmaxf(q0, 1e-12f));
    float devScale = 1.f / CD;
    float volGrad = J > .05f ? iso * I1 / (3.f * pJ) : 0.f;
    float CH = J - 1.f;
    f3 G[4], gd[4], gh[4];
#pragma unroll
    for (int c = 1; c < 4; c++) {
        f3 b = br[c - 1];
        gh[c] = fmv(cof[2], b.z, fmv(cof[1], b.y, cof[0] * b.x));
        G[c] = fmv(F[2], b.z, fmv(F[1], b.y, F[0] * b.x));
        gd[c] = fmv(G[c], iso, gh[c] * -volGrad) * devScale;
    }
    gd[0] = (gd[1] + gd[2] + gd[3]) * -1.f;
    gh[0] = (gh[1] + gh[2] + gh[3]) * -1.f;
    float dd = 0.f, dh = 0.f, vd = 0.f, vh = 0.f, w[4];
    f3 dx[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        w[c] = P[c].w;
        dd = fmaf(w[c], dotF(gd[c], gd[c]), dd);
        dh = fmaf(w[c], dotF(gd[c], gh[c]), dh);
        dx[c] = p[c] - q[c];
        vd += dotF(gd[c], dx[c]);
        vh += dotF(gh[c], dx[c]);
    }
    float scale = 1.f + dampingOverH, invScale = 1.f / scale;
    float eAd = ad * invScale, eAh = ah * invScale;
    float A = dd + eAd, invA = 1.f / A, Bc = dh, gamma = Bc * invA;
    float schur = fmaf(eAd * gamma, gamma, eAh);
    f3 r[4];
#pragma unroll
    for (int c = 0; c < 4; c++) { r[c] = fmv(gd[c], -gamma, gh[c]); schur = fmaf(w[c], dotF(r[c], r[c]), schur); }
    const bool damped = dampingOverH != 0.f;
    float rd = damped ? fmaf(-dampingOverH, vd, -CD) * invScale : -CD * invScale;
    float rh = damped ? fmaf(-(scale - 1.f), vh, -CH) * invScale : -CH * invScale;
    if (!(A > 0.f) || !(schur > 0.f)) return;
    float dlH = omega * fmaf(-gamma, rd, rh) / schur, dlD = fmaf(-Bc, dlH, omega * rd) * invA;
    if (!isfinite(dlD) || !isfinite(dlH)) return;
    // ---- reverse ----
    // o_c = p_c + (gd_c dlD + gh_c dlH) w_c
    f3 ggd[4], ggh[4];
    float gdlD = 0.f, gdlH = 0.f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        f3 gw = go[c] * w[c];
        ggd[c] = gw * dlD;
        ggh[c] = gw * dlH;
        gdlD += dot(gw, gd[c]);
        gdlH += dot(gw, gh[c]);
    }
    // dlD = (omega rd - Bc dlH) / A
    float t1 = gdlD * invA;
    float grd = omega * t1;
    float gBc = -(dlH * t1);
    gdlH = gdlH - Bc * t1;
    float gA = -(dlD * t1);
    // dlH = omega (rh - gamma rd) / schur
    float t2 = omega * gdlH / schur;
    float grh = t2;
    float ggamma = -(rd * t2);
    grd = grd - gamma * t2;
    float gschur = -(dlH * gdlH / schur);
    // rd = (-CD - D vd) / scale, rh = (-CH - (scale - 1) vh) / scale
    float ud = grd * invScale, uh = grh * invScale;
    float gCD = -ud, gvd = -(dampingOverH * ud);
    float gCH = -uh, gvh = -((scale - 1.f) * uh);
    // schur = eAh + eAd gamma^2 + sum w_c |gh_c - gd_c gamma|^2
    float geAh = gschur;
    float geAd = gamma * gamma * gschur;
    ggamma += 2.f * eAd * gamma * gschur;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        f3 gr = r[c] * (2.f * w[c] * gschur);
        ggh[c] = ggh[c] + gr;
        ggd[c] = ggd[c] - gr * gamma;
        ggamma -= dot(gr, gd[c]);
    }
    // gamma = Bc / A, A = dd + eAd, Bc = dh
    gBc += ggamma * invA;
    gA -= gamma * ggamma * invA;
    float gdd = gA, gdh = gBc;
    geAd += gA;
    // eAd = ad / scale, eAh = ah / scale
    out.gad = geAd * invScale;
    out.gah = geAh * invScale;
    // dd, dh, vd, vh
#pragma unroll
    for (int c = 0; c < 4; c++) {
        ggd[c] = ggd[c] + gd[c] * (2.f * w[c] * gdd) + gh[c] * (w[c] * gdh) + dx[c] * gvd;
        ggh[c] = ggh[c] + gd[c] * (w[c] * gdh) + dx[c] * gvh;
        f3 gdx = gd[c] * gvd + gh[c] * gvh;
        out.gp[c] = out.gp[c] + gdx;
        out.gq[c] = zero - gdx;
    }
    // gd_0 = -(gd_1 + gd_2 + gd_3), gh_0 likewise
#pragma unroll
    for (int c = 1; c < 4; c++) { ggd[c] = ggd[c] - ggd[0]; ggh[c] = ggh[c] - ggh[0]; }
    // gd_c = (G_c iso - gh_c volGrad) devScale, G_c = F b, gh_c = cof b  (b = row c-1 of Bm)
    f3 gF[3] = {zero, zero, zero}, gcof[3] = {zero, zero, zero};
    float giso = 0.f, gvolGrad = 0.f, gdevScale = 0.f;
#pragma unroll
    for (int c = 1; c < 4; c++) {
        f3 b = br[c - 1];
        f3 inner = G[c] * iso - gh[c] * volGrad;
        gdevScale += dot(ggd[c], inner);
        f3 gi = ggd[c] * devScale;
        giso += dot(gi, G[c]);
        gvolGrad -= dot(gi, gh[c]);
        f3 gG = gi * iso;
        ggh[c] = ggh[c] - gi * volGrad;
        gF[0] = gF[0] + gG * b.x; gF[1] = gF[1] + gG * b.y; gF[2] = gF[2] + gG * b.z;
        gcof[0] = gcof[0] + ggh[c] * b.x; gcof[1] = gcof[1] + ggh[c] * b.y; gcof[2] = gcof[2] + ggh[c] * b.z;
        if (wantB) {
            out.gB[3 * (c - 1) + 0] += dot(gG, F[0]) + dot(ggh[c], cof[0]);
            out.gB[3 * (c - 1) + 1] += dot(gG, F[1]) + dot(ggh[c], cof[1]);
            out.gB[3 * (c - 1) + 2] += dot(gG, F[2]) + dot(ggh[c], cof[2]);
        }
    }
    // CH = J - 1; volGrad = iso I1 / (3 pJ) where J > .05
    float gJ = gCH, gI1 = 0.f;
    if (J > .05f) {
        float den = 3.f * pJ;
        giso += gvolGrad * I1 / den;
        gI1 += gvolGrad * iso / den;
        gJ -= gvolGrad * volGrad / pJ;
    }
    // devScale = 1 / CD, CD = sqrt(max(q, 1e-12)), q = max(iso I1 - 3, 0)
    gCD -= gdevScale * devScale * devScale;
    if (q0 > 1e-12f) {
        float gq = gCD / (2.f * CD);
        giso += gq * I1;
        gI1 += gq * iso;
    }
    // iso = pJ^(-2/3), pJ = max(J, .05)
    if (J > .05f) gJ += giso * (-2.f / 3.f) * iso / pJ;
    // J = F_0 . (F_1 x F_2): dJ/dF_c = cof_c
#pragma unroll
    for (int c = 0; c < 3; c++) gF[c] = gF[c] + cof[c] * gJ + F[c] * (2.f * gI1);
    // cof_0 = F_1 x F_2, cof_1 = F_2 x F_0, cof_2 = F_0 x F_1
    gF[1] = gF[1] + cross(F[2], gcof[0]); gF[2] = gF[2] + cross(gcof[0], F[1]);
    gF[2] = gF[2] + cross(F[0], gcof[1]); gF[0] = gF[0] + cross(gcof[1], F[2]);
    gF[0] = gF[0] + cross(F[1], gcof[2]); gF[1] = gF[1] + cross(gcof[2], F[0]);
    // F_c = e_1 Bm[0][c] + e_2 Bm[1][c] + e_3 Bm[2][c], e_k = p_k - p_0
#pragma unroll
    for (int k = 0; k < 3; k++) {
        f3 ge = gF[0] * comp(br[k], 0) + gF[1] * comp(br[k], 1) + gF[2] * comp(br[k], 2);
        out.gp[k + 1] = out.gp[k + 1] + ge;
        out.gp[0] = out.gp[0] - ge;
        if (wantB) {
            out.gB[3 * k + 0] += dot(gF[0], e[k]);
            out.gB[3 * k + 1] += dot(gF[1], e[k]);
            out.gB[3 * k + 2] += dot(gF[2], e[k]);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// capsule contact (contact model 0, shaft branch; the differentiable rollout has no jaw)
// ---------------------------------------------------------------------------------------------
struct Capsule { f3 sa, sb; float radius, alpha; };

__device__ __forceinline__ f3 capsuleContact(f3 p, float wc, f3 v, const Capsule& k, const ContactParams& cp) {
    if (wc <= 0.f) return p;
    f3 ab = k.sb - k.sa;
    float ab2 = dot(ab, ab);
    float tt = ab2 > 1e-12f ? dot(p - k.sa, ab) / ab2 : 0.f;
    tt = fmaxf(0.f, fminf(1.f, tt));
    f3 dv = p - (k.sa + ab * tt);
    float dist = len(dv), C = dist - k.radius;
    if (C < 0.f) {
        f3 n = dist > 1e-9f ? dv * (1.f / dist) : mk(0.f, 1.f, 0.f);
        if (-dot(v, n) > cp.ccdVelThresh) {
            float dl = (-C - k.alpha * 0.f) / (wc + k.alpha);
            float ap = cp.ccdOmega * dl;
            f3 corr = n * (wc * ap);
            float cl = len(corr);
            if (cl > cp.ccdMaxDisp) { float s = cp.ccdMaxDisp / cl; corr = corr * s; }
            p = p + corr;
        }
    }
    return p;
}

// Adjoint of capsuleContact: returns the adjoint of p and adds the capsule end points' adjoints.
__device__ __forceinline__ f3 capsuleContactVJP(f3 p, float wc, f3 v, const Capsule& k, const ContactParams& cp, f3 go, f3& gsa,
                                                f3& gsb) {
    if (wc <= 0.f) return go;
    f3 ab = k.sb - k.sa;
    float ab2 = dot(ab, ab);
    float raw = ab2 > 1e-12f ? dot(p - k.sa, ab) / ab2 : 0.f;
    float tt = fmaxf(0.f, fminf(1.f, raw));
    f3 dv = p - (k.sa + ab * tt);
    float dist = len(dv), C = dist - k.radius;
    if (!(C < 0.f)) return go;
    bool normal = dist > 1e-9f;
    float inv = normal ? 1.f / dist : 0.f;
    f3 n = normal ? dv * inv : mk(0.f, 1.f, 0.f);
    if (!(-dot(v, n) > cp.ccdVelThresh)) return go;
    float den = wc + k.alpha;
    float dl = (-C - k.alpha * 0.f) / den;
    float ap = cp.ccdOmega * dl;
    f3 corr0 = n * (wc * ap);
    float cl = len(corr0);
    f3 gcorr0 = go;
    if (cl > cp.ccdMaxDisp) {   // corr = corr0 maxDisp / |corr0|
        float s = cp.ccdMaxDisp / cl;
        gcorr0 = go * s - corr0 * (dot(go, corr0) * s / (cl * cl));
    }
    f3 gp = go;
    // corr0 = n (wc ap), ap = omega dl, dl = -C / den, C = dist - r
    f3 gn = gcorr0 * (wc * ap);
    float gap = wc * dot(gcorr0, n);
    float gdist = -(cp.ccdOmega * gap / den);
    f3 gdv = mk(0.f, 0.f, 0.f);
    if (normal) {   // n = dv inv, dist = |dv|
        gdist -= dot(gn, dv) * (inv * inv);
        gdv = gn * inv + n * gdist;
    }
    gp = gp + gdv;
    // dv = p - (sa + ab tt)
    gsa = gsa - gdv;
    f3 gab = gdv * -tt;
    float gtt = -dot(gdv, ab);
    if (ab2 > 1e-12f && raw > 0.f && raw < 1.f) {   // raw = (p - sa).ab / ab2
        f3 g1 = ab * (gtt / ab2);
        gp = gp + g1;
        gsa = gsa - g1;
        gab = gab + (p - k.sa) * (gtt / ab2) - ab * (2.f * gtt * raw / ab2);
    }
    gsb = gsb + gab;
    gsa = gsa - gab;
    return gp;
}

}  // namespace gbt
