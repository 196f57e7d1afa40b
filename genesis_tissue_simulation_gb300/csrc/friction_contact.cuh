// Contact model 1 on lattice nodes: finite tool SDFs, swept contact and unilateral Coulomb friction
// (V/contact/friction_contact.cuh:3-169, dispatched at V/xpbd/xpbd_solver.cu:3655-3665 when no
// reconstructed surface exists).
//
// Per substep the instrument gives three shapes — the shaft capsule and two jaw boxes opened by the
// jaw gap — at the previous and the current interpolation parameter.  Each lattice node traces its
// motion over the substep against each shape: an exact piecewise-quadratic time of impact for a
// translating box, conservative advancement in double-precision time otherwise (it terminates: the
// parameter grows by at least 0.8 tol / speed per step).  Then two Gauss-Jacobi passes project the
// unilateral normal constraint and Coulomb friction per node.  Nodes are independent, so the whole
// model is one node-parallel phase.  Scalars follow the reference's types: geometry in float, the
// time of impact in double.
#pragma once
#include "tissue_device.cuh"

namespace gbt {

struct CShape { f3 center, u, n, w, half, a, b; float radius; int capsule; };
struct CRecord { f3 normal, target, motion; int valid; };

__device__ __forceinline__ f3 cUnit(f3 x, f3 fallback) { float l = len(x); return l > 1e-8f ? x * (1.f / l) : fallback; }

__device__ __forceinline__ CShape cShape(f3 hinge, f3 axis, f3 normalIn, f3 shaftA, f3 shaftB, float shaftR, float jawGap, float jawLen,
                                         float halfWidth, int kind, float thickness, float minGap) {
    CShape s = {};
    s.capsule = kind == 0;
    if (kind == 0) { s.a = shaftA; s.b = shaftB; s.radius = shaftR; return s; }
    f3 u = cUnit(axis, mk(0.f, 0.f, 1.f));
    f3 n = normalIn - u * dot(u, normalIn);
    n = cUnit(n, fabsf(u.y) < .9f ? cUnit(cross(u, mk(0.f, 1.f, 0.f)), mk(1.f, 0.f, 0.f)) : mk(1.f, 0.f, 0.f));
    float side = kind == 1 ? 1.f : -1.f;
    float sn = fminf(.95f, fmaxf(0.f, jawGap) / (2.f * fmaxf(jawLen, 1e-6f)));
    float cs = sqrtf(1.f - sn * sn);
    s.u = u * cs + n * (side * sn); s.n = n * cs - u * (side * sn); s.w = cross(s.u, s.n);
    s.half = mk(jawLen * .5f, thickness * .5f, halfWidth);
    s.center = hinge + s.u * s.half.x + s.n * (side * (s.half.y + .5f * minGap));
    return s;
}

__device__ __forceinline__ float cDistance(const CShape& s, f3 x, f3& normal, f3& surface) {
    if (s.capsule) {
        f3 ab = s.b - s.a;
        float tt = fminf(1.f, fmaxf(0.f, dot(x - s.a, ab) / fmaxf(dot(ab, ab), 1e-20f)));
        f3 d = x - (s.a + ab * tt);
        float l = len(d);
        f3 fallback = cUnit(cross(ab, fabsf(ab.x) < fabsf(ab.y) ? mk(1.f, 0.f, 0.f) : mk(0.f, 1.f, 0.f)), mk(0.f, 0.f, 1.f));
        normal = l > 1e-6f * fmaxf(1.f, len(ab)) ? d * (1.f / l) : fallback;
        surface = s.a + ab * tt + normal * s.radius;
        return l - s.radius;
    }
    f3 r = x - s.center;
    float v[3] = {dot(r, s.u), dot(r, s.n), dot(r, s.w)};
    float h[3] = {s.half.x, s.half.y, s.half.z}, q[3], cl[3];
#pragma unroll
    for (int k = 0; k < 3; k++) { q[k] = fabsf(v[k]) - h[k]; cl[k] = fminf(h[k], fmaxf(-h[k], v[k])); }
    f3 closest = s.center + s.u * cl[0] + s.n * cl[1] + s.w * cl[2];
    f3 d = s.u * copysignf(fmaxf(q[0], 0.f), v[0]) + s.n * copysignf(fmaxf(q[1], 0.f), v[1]) + s.w * copysignf(fmaxf(q[2], 0.f), v[2]);
    float dl = len(d);
    if (q[0] > 0.f || q[1] > 0.f || q[2] > 0.f) { normal = dl > 0.f ? d * (1.f / dl) : s.n; surface = closest; return dl; }
    int k = q[1] > q[0] ? 1 : 0;
    if (q[2] > q[k]) k = 2;
    f3 ax = k == 0 ? s.u : (k == 1 ? s.n : s.w);
    normal = ax * (v[k] >= 0.f ? 1.f : -1.f);
    surface = x - normal * q[k];
    return q[k];
}

__device__ __forceinline__ CShape cLerp(const CShape& a, const CShape& b, float t) {
    CShape s = b;
    s.center = a.center * (1.f - t) + b.center * t;
    s.a = a.a * (1.f - t) + b.a * t;
    s.b = a.b * (1.f - t) + b.b * t;
    s.u = cUnit(a.u * (1.f - t) + b.u * t, b.u);
    s.n = a.n * (1.f - t) + b.n * t;
    s.n = cUnit(s.n - s.u * dot(s.u, s.n), b.n);
    s.w = cross(s.u, s.n);
    return s;
}

__device__ __forceinline__ f3 cRotateShaft(const CShape& from, const CShape& to, f3 r) {
    f3 a = from.b - from.a, b = to.b - to.a;
    if (len(a) < 1e-8f || len(b) < 1e-8f) return r;
    a = cUnit(a, mk(0.f, 0.f, 1.f));
    b = cUnit(b, a);
    float c = fminf(1.f, fmaxf(-1.f, dot(a, b)));
    f3 v = cross(a, b);
    if (c < -.9999f) {
        f3 u = cUnit(cross(a, fabsf(a.x) < .9f ? mk(1.f, 0.f, 0.f) : mk(0.f, 1.f, 0.f)), mk(0.f, 0.f, 1.f));
        return u * (2.f * dot(u, r)) - r;
    }
    return r + cross(v, r) + cross(v, cross(v, r)) * (1.f / (1.f + c));
}

__device__ __forceinline__ f3 cWitness(const CShape& from, const CShape& to, f3 p) {
    if (from.capsule) {
        f3 ab = from.b - from.a;
        float t = fminf(1.f, fmaxf(0.f, dot(p - from.a, ab) / fmaxf(dot(ab, ab), 1e-20f)));
        return to.a + (to.b - to.a) * t + cRotateShaft(from, to, p - from.a - ab * t);
    }
    f3 r = p - from.center;
    return to.center + to.u * dot(r, from.u) + to.n * dot(r, from.n) + to.w * dot(r, from.w);
}

__device__ __forceinline__ bool cPointBoxTime(const CShape& box, float radius, f3 a, f3 b, float& time) {
    f3 axes[3] = {box.u, box.n, box.w};
    float p[3], v[3], half[3], cuts[8] = {0.f, 1.f};
    int count = 2;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p[k] = dot(a, axes[k]); v[k] = dot(b - a, axes[k]); half[k] = comp(box.half, k);
        if (fabsf(v[k]) > 1e-12f)
            for (int side = -1; side <= 1; side += 2) {
                float t = ((float)side * half[k] - p[k]) / v[k];
                if (t > 0.f && t < 1.f) cuts[count++] = t;
            }
    }
    for (int i = 1; i < count; i++) {
        float x = cuts[i];
        int j = i;
        while (j > 0 && cuts[j - 1] > x) { cuts[j] = cuts[j - 1]; --j; }
        cuts[j] = x;
    }
    for (int i = 0; i < count - 1; i++) {
        double A = 0, B = 0, C = -(double)radius * radius;
        float lo = cuts[i], hi = cuts[i + 1], mid = .5f * (lo + hi);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float q = p[k] + v[k] * mid;
            if (fabsf(q) <= half[k]) continue;
            double d = p[k] - copysignf(half[k], q);
            A += (double)v[k] * v[k]; B += 2 * d * v[k]; C += d * d;
        }
        double atLo = (A * lo + B) * lo + C;
        if (atLo <= 1e-14) { time = lo; return true; }
        if (A <= 1e-24) continue;
        double disc = B * B - 4 * A * C;
        if (disc < 0) continue;
        double root = (-B - sqrt(disc)) / (2 * A);
        if (root >= lo - 1e-8 && root <= hi + 1e-8) { time = fminf(hi, fmaxf(lo, (float)root)); return true; }
    }
    return false;
}

__device__ __noinline__ CRecord cTrace(const CShape& from, const CShape& to, float radius, f3 x0, f3 x1) {
    CRecord out = {};
    f3 normal = mk(0.f, 0.f, 0.f), surface = mk(0.f, 0.f, 0.f);
    if (!to.capsule && len(to.u - from.u) + len(to.n - from.n) < 1e-7f) {
        float time = 0.f;
        if (!cPointBoxTime(to, radius, x0 - from.center, x1 - to.center, time)) return out;
        CShape hit = cLerp(from, to, time);
        cDistance(hit, x0 * (1.f - time) + x1 * time, normal, surface);
        f3 end = cWitness(hit, to, surface), start = cWitness(hit, from, surface);
        out.normal = normal; out.target = end + normal * radius; out.motion = end - start; out.valid = 1;
        return out;
    }
    float speed = len(x1 - x0);
    if (to.capsule) speed += fmaxf(len(to.a - from.a), len(to.b - from.b));
    else speed += len(to.center - from.center) + 4.f * len(to.half) * (len(to.u - from.u) + len(to.n - from.n));
    f3 center0 = to.capsule ? (from.a + from.b) * .5f : from.center;
    f3 center1 = to.capsule ? (to.a + to.b) * .5f : to.center;
    float bound = to.capsule ? fmaxf(len(from.b - from.a), len(to.b - to.a)) * .5f + to.radius : len(to.half);
    if (len(x0 - center0) > bound + radius + len(x1 - x0) + len(center1 - center0) + 1e-5f) return out;
    float tol = fmaxf(1e-6f, 1e-4f * (bound + radius));
    double t = 0;
    CShape hit = from;
    bool found = false;
    while (t < 1.) {
        hit = cLerp(from, to, (float)t);
        float d = cDistance(hit, x0 * (float)(1 - t) + x1 * (float)t, normal, surface) - radius;
        if (d <= tol) { found = true; break; }
        if (speed <= 1e-12f) break;
        float step = .8f * d / speed;
        if (t + step >= 1.f) {
            t = 1; hit = to;
            float de = cDistance(to, x1, normal, surface) - radius;
            found = de <= tol;
            break;
        }
        t += step;
    }
    if (!found) return out;
    f3 end = cWitness(hit, to, surface), start = cWitness(hit, from, surface);
    if (to.capsule) normal = cRotateShaft(hit, to, normal);
    else normal = cUnit(to.u * dot(normal, hit.u) + to.n * dot(normal, hit.n) + to.w * dot(normal, hit.w), normal);
    out.normal = normal; out.target = end + normal * radius; out.motion = end - start; out.valid = 1;
    return out;
}

// The six shapes of one substep: [0..2] at the previous parameter, [3..5] at the current one.
struct FrictionShapes { CShape s[6]; };
__device__ __forceinline__ FrictionShapes frictionShapes(const ToolPose& a, const ToolPose& b, float t, float previousT, float thickness,
                                                         float minGap) {
    FrictionShapes f;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        float u = k == 0 ? previousT : t;
        f3 hinge = lerpTool(a.hx, a.hy, a.hz, b.hx, b.hy, b.hz, u), axis = lerpTool(a.ax, a.ay, a.az, b.ax, b.ay, b.az, u);
        f3 nrm = lerpTool(a.nx, a.ny, a.nz, b.nx, b.ny, b.nz, u);
        f3 sa = lerpTool(a.sax, a.say, a.saz, b.sax, b.say, b.saz, u), sb = lerpTool(a.sbx, a.sby, a.sbz, b.sbx, b.sby, b.sbz, u);
        float gap = a.gap * (1.f - u) + b.gap * u;
        for (int kind = 0; kind < 3; kind++)
            f.s[3 * k + kind] = cShape(hinge, axis, nrm, sa, sb, b.shaftR, gap, b.len, b.halfWidth, kind, thickness, minGap);
    }
    return f;
}

// Contact model 1 for one node (k_FindToolContacts x 3 shapes, then k_SolveFrictionContacts x 2).
__device__ __noinline__ void frictionNode(const DeviceMesh& m, int i, const FrictionShapes& f, float radius, float alpha, float muS,
                                          float muD) {
    float4 P = m.pos[i];
    float w = P.w;
    if (!(w > 0.f)) return;
    f3 x = xyz(P), q = xyz(m.prev[i]);
    CRecord rec[3];
    for (int kind = 0; kind < 3; kind++) {
        const CShape& to = f.s[3 + kind];
        rec[kind] = CRecord{};
        if (to.capsule ? to.radius > 0.f : (to.half.x > 0.f && to.half.z > 0.f)) rec[kind] = cTrace(f.s[kind], to, radius, q, x);
    }
    float lambdaN[3] = {0.f, 0.f, 0.f};
    f3 lambdaT[3] = {mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f)};
    for (int it = 0; it < 2; it++)
        for (int kind = 0; kind < 3; kind++) {
            const CRecord& c = rec[kind];
            if (!c.valid) continue;
            float C = dot(x - c.target, c.normal), old = lambdaN[kind];
            float next = fmaxf(0.f, old + (-C - alpha * old) / (w + alpha));
            x = x + c.normal * (w * (next - old));
            lambdaN[kind] = next;
            f3 slip = x - q - c.motion;
            slip = slip - c.normal * dot(slip, c.normal);
            f3 oldT = lambdaT[kind], trial = oldT - slip * (1.f / w);
            float tl = len(trial);
            f3 nextT = trial;
            if (tl > muS * next) nextT = tl > 1e-15f ? trial * (muD * next / tl) : mk(0.f, 0.f, 0.f);
            x = x + (nextT - oldT) * w;
            lambdaT[kind] = nextT;
        }
    m.pos[i] = make_float4(x.x, x.y, x.z, w);
}

}  // namespace gbt
