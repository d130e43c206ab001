// ffsrl_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of FF-SRL's multi-environment step, BVH refit and ray-cast
// (reference: FF_SRL/FF_SRL/integrator.py, bvh.py, render.py, utils.py).  It is the
// checker for libffsrl_cuda.so and the timed CPU baseline; nothing in the product links,
// loads or calls it.  Kernels run serially in reference launch order and thread-id
// order, which is what Warp's CPU backend does with one thread per launch.
//
// Parity status: the reference cannot run here (warp-lang 0.10.1 and pxr are absent)
// and ships no golden vectors, so this restatement is pinned by the known-answer tests
// in tests/ (single constraints with analytic answers, hand-built BVHs, a ray at a
// unit triangle) rather than by reference outputs.
//
// Arithmetic follows the reference expression by expression (same association order,
// float32 unless templated to double).  Build with -ffp-contract=off so no multiply-add
// is fused.  Warp built-ins are defined from their mathematics:
//   length(v) = sqrt(dot(v,v)), dot = (x*x' + y*y') + z*z',
//   normalize(v) = v/|v| if |v| > 0 else 0,
//   min/max(a,b) = a<b?a:b / a>b?a:b (component-wise),
//   quat_rotate(q,v) = v*(2w^2-1) + q.xyz*(2 q.xyz.v) + cross(q.xyz,v)*(2w).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include "../include/ffsrl.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// FLOAT_EPSILON = sys.float_info.epsilon (integrator.py:8), used in float32 comparisons.
const double kFloatEpsilon = 2.220446049250313e-16;

template <class R> struct V3 { R x, y, z; };
template <class R> inline V3<R> mk(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return mk<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return mk<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> inline V3<R> operator-(V3<R> a) { return mk<R>(-a.x, -a.y, -a.z); }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return mk<R>(a.x * s, a.y * s, a.z * s); }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return mk<R>(s * a.x, s * a.y, s * a.z); }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return mk<R>(a.x / s, a.y / s, a.z / s); }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return mk<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a) {
    R l = length(a);
    if (l > R(0)) return a / l;
    return mk<R>(0, 0, 0);
}
template <class R> inline R rmin(R a, R b) { return a < b ? a : b; }
template <class R> inline R rmax(R a, R b) { return a > b ? a : b; }
template <class R> inline V3<R> vmin(V3<R> a, V3<R> b) { return mk<R>(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)); }
template <class R> inline V3<R> vmax(V3<R> a, V3<R> b) { return mk<R>(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); }

template <class R, class S> inline V3<R> ld3(const S* p, int64_t i) {
    return mk<R>(R(p[3 * i]), R(p[3 * i + 1]), R(p[3 * i + 2]));
}
template <class R, class S> inline void st3(S* p, int64_t i, V3<R> v) {
    p[3 * i] = S(v.x); p[3 * i + 1] = S(v.y); p[3 * i + 2] = S(v.z);
}

// ----------------------------------------------------------------------------------
// Simulation state in precision R.  Constants stay in the model's float arrays and are
// promoted on read.
template <class R> struct Sim {
    const ffsrl_model* m;
    const ffsrl_params* p;
    std::vector<R> x, xp, v, dp, cdp, tlam, elam;
    std::vector<int32_t> cnt;
    std::vector<int32_t> incol;
    R dt, eps;
};

// gravity (integrator.py:40-63)
template <class R> void k_gravity(Sim<R>& s, int64_t i) {
    const ffsrl_params* p = s.p;
    V3<R> x = ld3<R>(s.x.data(), i);
    V3<R> v = ld3<R>(s.v.data(), i);
    R inv = R(s.m->inverse_mass[i]);
    R damp = R(1) - R(p->velocity_dampening);
    V3<R> g = mk<R>(R(p->gravity[0]), R(p->gravity[1]), R(p->gravity[2]));
    v = v + g * inv * s.dt * damp;
    if (inv < R(kFloatEpsilon)) v = mk<R>(0, 0, 0);
    st3(s.xp.data(), i, x + v * s.dt);
}

// volumeConstraints (integrator.py:444-504)
template <class R> void k_volume(Sim<R>& s, int64_t t) {
    const ffsrl_model* m = s.m;
    R active = R(m->active_tetrahedron[t]);
    if (!(active == R(1))) return;
    int a = m->tetrahedron[4 * t], b = m->tetrahedron[4 * t + 1], c = m->tetrahedron[4 * t + 2], d = m->tetrahedron[4 * t + 3];
    V3<R> pa = ld3<R>(s.xp.data(), a), pb = ld3<R>(s.xp.data(), b), pc = ld3<R>(s.xp.data(), c), pd = ld3<R>(s.xp.data(), d);
    R rv = R(m->tetrahedron_rest_volume[t]);
    V3<R> p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
    V3<R> q2 = cross(p3, p1), q1 = cross(p2, p3), q3 = cross(p1, p2);
    V3<R> q0 = -q1 - q2 - q3;
    R mA = R(m->inverse_mass[a]), mB = R(m->inverse_mass[b]), mC = R(m->inverse_mass[c]), mD = R(m->inverse_mass[d]);
    R vol = std::fabs(dot(cross(p1, p2), p3)) / R(6);
    R w = mA * dot(q0, q0) + mB * dot(q1, q1) + mC * dot(q2, q2) + mD * dot(q3, q3);
    if (std::fabs(w) < R(kFloatEpsilon)) return;
    R C = rv - vol;
    R dl = -R(s.p->ks_volume) * active * C / w;
    auto add = [&](int vi, V3<R> dv) {
        s.dp[3 * vi] += dv.x; s.dp[3 * vi + 1] += dv.y; s.dp[3 * vi + 2] += dv.z; s.cnt[vi] += 1;
    };
    add(a, q0 * dl * mA); add(b, q1 * dl * mB); add(c, q2 * dl * mC); add(d, q3 * dl * mD);
}

// volumeConstraintsXPBD (integrator.py:507-576); rest volume is signed
template <class R> void k_volume_xpbd(Sim<R>& s, int64_t t, R alpha) {
    const ffsrl_model* m = s.m;
    if (!(R(m->active_tetrahedron[t]) == R(1))) return;
    int a = m->tetrahedron[4 * t], b = m->tetrahedron[4 * t + 1], c = m->tetrahedron[4 * t + 2], d = m->tetrahedron[4 * t + 3];
    V3<R> pa = ld3<R>(s.xp.data(), a), pb = ld3<R>(s.xp.data(), b), pc = ld3<R>(s.xp.data(), c), pd = ld3<R>(s.xp.data(), d);
    R rv = R(m->xpbd_rest_volume[t]);
    R lam = s.tlam[t];
    V3<R> p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
    V3<R> q2 = cross(p3, p1), q1 = cross(p2, p3), q3 = cross(p1, p2);
    V3<R> q0 = -q1 - q2 - q3;
    R mA = R(m->inverse_mass[a]), mB = R(m->inverse_mass[b]), mC = R(m->inverse_mass[c]), mD = R(m->inverse_mass[d]);
    R vol = dot(cross(p1, p2), p3) / R(6);
    R w = mA * dot(q0, q0) + mB * dot(q1, q1) + mC * dot(q2, q2) + mD * dot(q3, q3);
    if (std::fabs(w) < R(kFloatEpsilon)) return;
    R C = vol - rv;
    R dl = -(C + alpha * lam) / (w + alpha);
    s.tlam[t] = lam + dl;
    auto add = [&](int vi, V3<R> dv) {
        s.dp[3 * vi] += dv.x; s.dp[3 * vi + 1] += dv.y; s.dp[3 * vi + 2] += dv.z; s.cnt[vi] += 1;
    };
    add(a, q0 * dl * mA); add(b, q1 * dl * mB); add(c, q2 * dl * mC); add(d, q3 * dl * mD);
}

// neoHookeanConstraints (integrator.py:578-698), Macklin-Mueller stable Neo-Hookean.
// F = Ds * Dm^-1 with Ds = [p1 p2 p3] as columns; the gradient for vertex i (1..3) is
// column i of dC/dF * Dm^-T; vertex A gets minus their sum.  The reference's lambda
// is a local (never stored), so each projection starts from lambda = 0.
template <class R> void k_neohookean(Sim<R>& s, int64_t t) {
    const ffsrl_model* m = s.m;
    int a = m->tetrahedron[4 * t], b = m->tetrahedron[4 * t + 1], c = m->tetrahedron[4 * t + 2], d = m->tetrahedron[4 * t + 3];
    R rv = R(m->tetrahedron_rest_volume[t]);
    V3<R> pa = ld3<R>(s.xp.data(), a), pb = ld3<R>(s.xp.data(), b), pc = ld3<R>(s.xp.data(), c), pd = ld3<R>(s.xp.data(), d);
    V3<R> p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
    R mA = R(m->inverse_mass[a]), mB = R(m->inverse_mass[b]), mC = R(m->inverse_mass[c]), mD = R(m->inverse_mass[d]);
    const float* D = m->tetrahedron_dm_inv + 9 * t;
    R Dm[3][3];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) Dm[r][q] = R(D[3 * r + q]);
    // columns of F
    V3<R> f0 = p1 * Dm[0][0] + p2 * Dm[1][0] + p3 * Dm[2][0];
    V3<R> f1 = p1 * Dm[0][1] + p2 * Dm[1][1] + p3 * Dm[2][1];
    V3<R> f2 = p1 * Dm[0][2] + p2 * Dm[1][2] + p3 * Dm[2][2];
    // hydrostatic: dC/dF = cof(F), columns f1xf2, f2xf0, f0xf1
    V3<R> c0 = cross(f1, f2), c1 = cross(f2, f0), c2 = cross(f0, f1);
    V3<R> g1 = c0 * Dm[0][0] + c1 * Dm[0][1] + c2 * Dm[0][2];
    V3<R> g2 = c0 * Dm[1][0] + c1 * Dm[1][1] + c2 * Dm[1][2];
    V3<R> g3 = c0 * Dm[2][0] + c1 * Dm[2][1] + c2 * Dm[2][2];
    V3<R> g0 = -g1 - g2 - g3;
    R detF = dot(f0, c0);
    R invVol = R(1) / R(s.p->volume_compliance);
    R invDev = R(1) / R(s.p->deviatoric_compliance);
    R C = detF - R(1) - invDev / invVol;
    R w = R(0);
    R l;
    l = length(g0); w += l * l * mA;
    l = length(g1); w += l * l * mB;
    l = length(g2); w += l * l * mC;
    l = length(g3); w += l * l * mD;
    if (w < R(kFloatEpsilon)) return;
    R alpha = R(s.p->volume_compliance) / s.dt / s.dt / rv;
    R dl = -C / (w + alpha);
    V3<R> dA = g0 * dl * mA, dB = g1 * dl * mB, dC = g2 * dl * mC, dD = g3 * dl * mD;
    // deviatoric: C = ||F||_F, dC/dF = F / ||F||_F
    R l0 = length(f0), l1 = length(f1), l2 = length(f2);
    R rs = std::sqrt(l0 * l0 + l1 * l1 + l2 * l2);
    R rsi = R(1) / rs;
    C = rs;
    g1 = (f0 * Dm[0][0] + f1 * Dm[0][1] + f2 * Dm[0][2]) * rsi;
    g2 = (f0 * Dm[1][0] + f1 * Dm[1][1] + f2 * Dm[1][2]) * rsi;
    g3 = (f0 * Dm[2][0] + f1 * Dm[2][1] + f2 * Dm[2][2]) * rsi;
    g0 = -g1 - g2 - g3;
    w = R(0);
    l = length(g0); w += l * l * mA;
    l = length(g1); w += l * l * mB;
    l = length(g2); w += l * l * mC;
    l = length(g3); w += l * l * mD;
    if (w < R(kFloatEpsilon)) return;
    alpha = R(s.p->deviatoric_compliance) / s.dt / s.dt / rv;
    dl = -C / (w + alpha);
    dA = dA + g0 * dl * mA; dB = dB + g1 * dl * mB; dC = dC + g2 * dl * mC; dD = dD + g3 * dl * mD;
    auto add = [&](int vi, V3<R> dv) {
        s.dp[3 * vi] += dv.x; s.dp[3 * vi + 1] += dv.y; s.dp[3 * vi + 2] += dv.z; s.cnt[vi] += 1;
    };
    add(a, dA); add(b, dB); add(c, dC); add(d, dD);
}

// distanceConstraints (integrator.py:65-109)
template <class R> void k_distance(Sim<R>& s, int64_t e) {
    const ffsrl_model* m = s.m;
    R active = R(m->active_edge[e]);
    if (active == R(0)) return;
    int a = m->edge[2 * e], b = m->edge[2 * e + 1];
    V3<R> pa = ld3<R>(s.xp.data(), a), pb = ld3<R>(s.xp.data(), b);
    R L0 = R(m->edge_rest_length[e]);
    if (L0 < R(kFloatEpsilon)) return;
    V3<R> dir = pb - pa;
    R len = length(dir);
    if (len < R(kFloatEpsilon)) return;
    R mA = R(m->inverse_mass[a]), mB = R(m->inverse_mass[b]);
    R w = mA + mB;
    if (w < R(kFloatEpsilon)) return;
    R C = len - L0;
    V3<R> d = -C * (dir / len) * R(s.p->ks_distance) * active / w;
    V3<R> da = d * mA, db = d * mB;
    s.dp[3 * a] -= da.x; s.dp[3 * a + 1] -= da.y; s.dp[3 * a + 2] -= da.z;
    s.dp[3 * b] += db.x; s.dp[3 * b + 1] += db.y; s.dp[3 * b + 2] += db.z;
    s.cnt[a] += 1; s.cnt[b] += 1;
}

// distanceConstraintsXPBD (integrator.py:191-240)
template <class R> void k_distance_xpbd(Sim<R>& s, int64_t e, R alpha) {
    const ffsrl_model* m = s.m;
    if (R(m->active_edge[e]) == R(0)) return;
    int a = m->edge[2 * e], b = m->edge[2 * e + 1];
    V3<R> pa = ld3<R>(s.xp.data(), a), pb = ld3<R>(s.xp.data(), b);
    R L0 = R(m->edge_rest_length[e]);
    if (L0 < R(kFloatEpsilon)) return;
    R lam = s.elam[e];
    V3<R> dir = pb - pa;
    R len = length(dir);
    if (len < R(kFloatEpsilon)) return;
    R mA = R(m->inverse_mass[a]), mB = R(m->inverse_mass[b]);
    R w = mA + mB;
    if (w < R(kFloatEpsilon)) return;
    R C = len - L0;
    R dl = -(C + alpha * lam) / (w + alpha);
    s.elam[e] = lam + dl;
    V3<R> d = dl * normalize(dir);
    V3<R> da = d * mA, db = d * mB;
    s.dp[3 * a] -= da.x; s.dp[3 * a + 1] -= da.y; s.dp[3 * a + 2] -= da.z;
    s.dp[3 * b] += db.x; s.dp[3 * b + 1] += db.y; s.dp[3 * b + 2] += db.z;
    s.cnt[a] += 1; s.cnt[b] += 1;
}

// applyConstraints (integrator.py:946-960)
template <class R> void k_apply(Sim<R>& s, int64_t i) {
    if (s.cnt[i] > 0) {
        R n = R(s.cnt[i]);
        V3<R> dp = ld3<R>(s.dp.data(), i);
        V3<R> x = ld3<R>(s.xp.data(), i);
        st3(s.xp.data(), i, x + mk<R>(dp.x / n, dp.y / n, dp.z / n));
    }
    s.dp[3 * i] = s.dp[3 * i + 1] = s.dp[3 * i + 2] = R(0);
    s.cnt[i] = 0;
}

// dragConstraintsDO (integrator.py:412-442): pulls toward laparoscopeTip[env*4 + 2]
template <class R> void k_drag(Sim<R>& s, int64_t i) {
    const ffsrl_model* m = s.m;
    R drag = R(m->active_drag_constraint[i]);
    int env = m->vertex_to_env[i];
    if (drag == R(0)) return;
    V3<R> pos = ld3<R>(s.xp.data(), i);
    V3<R> tip = ld3<R>(m->laparoscope_tip, int64_t(env) * 4 + 2);
    V3<R> dir = pos - tip;
    R len = length(dir);
    if (len < R(kFloatEpsilon)) return;
    R inv = R(2);
    V3<R> d = len * normalize(dir) * drag * R(s.p->ks_drag) / inv;
    st3(s.xp.data(), i, pos - d);
}

// triToPointDistanceConstraintsDO (integrator.py:300-353)
template <class R> void k_connector(Sim<R>& s, int64_t c) {
    const ffsrl_model* m = s.m;
    const ffsrl_params* p = s.p;
    int ta = m->connector_triangle_id[3 * c], tb = m->connector_triangle_id[3 * c + 1], tc = m->connector_triangle_id[3 * c + 2];
    V3<R> A = ld3<R>(s.xp.data(), ta), B = ld3<R>(s.xp.data(), tb), Cc = ld3<R>(s.xp.data(), tc);
    V3<R> bar = ld3<R>(m->connector_tri_bar, c);
    V3<R> centre = A * bar.x + B * bar.y + Cc * bar.z;
    int pid = m->connector_vertex_id[c];
    V3<R> pos = ld3<R>(s.xp.data(), pid);
    R rd = R(m->connector_rest_dist[c]);
    V3<R> dir = pos - centre;
    R len = length(dir);
    if (len < R(kFloatEpsilon)) return;
    R wp = R(p->connector_mass_weight_ratio);
    R wt = R(1) - wp;
    R C = len - rd * R(p->connector_rest_length_mul);
    R sden = wp + wt * (bar.x * bar.x + bar.y * bar.y + bar.z * bar.z);
    V3<R> delta = (C / sden) * (dir / len) * R(p->connector_ks);
    auto add = [&](int vi, V3<R> dv) { s.dp[3 * vi] += dv.x; s.dp[3 * vi + 1] += dv.y; s.dp[3 * vi + 2] += dv.z; };
    add(pid, -(delta * wp));
    add(ta, delta * wt * bar.x);
    add(tb, delta * wt * bar.y);
    add(tc, delta * wt * bar.z);
    s.cnt[pid] += 1; s.cnt[ta] += 1; s.cnt[tb] += 1; s.cnt[tc] += 1;
}

// closestPointOnEdge (integrator.py:1520-1534)
template <class R> V3<R> closest_on_edge(V3<R> p, V3<R> a, V3<R> b) {
    V3<R> d = b - a;
    R t;
    if (length(d) < R(kFloatEpsilon)) {
        t = R(0.5);
    } else {
        R ld = length(d);
        R d2 = ld * ld;
        t = dot(d, p - a) / d2;
        if (t < R(0)) t = R(0);
        else if (t > R(1)) t = R(1);
    }
    return a + d * t;
}

// triangle_closest_point_barycentric (integrator.py:1536-1581)
template <class R> V3<R> closest_bary(V3<R> a, V3<R> b, V3<R> c, V3<R> p) {
    V3<R> ab = b - a, ac = c - a, ap = p - a;
    R d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= R(0) && d2 <= R(0)) return mk<R>(1, 0, 0);
    V3<R> bp = p - b;
    R d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= R(0) && d4 <= d3) return mk<R>(0, 1, 0);
    R vc = d1 * d4 - d3 * d2;
    R v = d1 / (d1 - d3);
    if (vc <= R(0) && d1 >= R(0) && d3 <= R(0)) return mk<R>(R(1) - v, v, 0);
    V3<R> cp = p - c;
    R d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= R(0) && d5 <= d6) return mk<R>(0, 0, 1);
    R vb = d5 * d2 - d1 * d6;
    R w = d2 / (d2 - d6);
    if (vb <= R(0) && d2 >= R(0) && d6 <= R(0)) return mk<R>(R(1) - w, 0, w);
    R va = d3 * d6 - d5 * d4;
    w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    if (va <= R(0) && (d4 - d3) >= R(0) && (d5 - d6) >= R(0)) return mk<R>(0, w, R(1) - w);
    R denom = R(1) / (va + vb + vc);
    v = vb * denom;
    w = vc * denom;
    return mk<R>(R(1) - v - w, v, w);
}

// checkSdfCapsuleCollision (integrator.py:1302-1355); returns true with the three
// vertex responses when in contact
template <class R> bool capsule_response(V3<R> tip, V3<R> base, R radius, V3<R> n, V3<R> centre,
                                         V3<R> pA, V3<R> pB, V3<R> pC, R ks, V3<R>* out) {
    V3<R> cn = normalize(tip - base);
    V3<R> off = cn * radius;
    V3<R> posA = base + off;
    V3<R> posB = tip - off;
    R denom = dot(n, cn);
    if (std::fabs(denom) < R(kFloatEpsilon)) return false;
    R t = dot(n, centre - base) / denom;
    V3<R> lp = base + cn * t;
    V3<R> ref = closest_bary(pA, pB, pC, lp);
    V3<R> refp = ref;  // referencePoint is the barycentric vec3 itself (integrator.py:1330)
    V3<R> sc = closest_on_edge(refp, posA, posB);
    V3<R> bary = closest_bary(pA, pB, pC, sc);
    V3<R> contact = pA * bary.x + pB * bary.y + pC * bary.z;
    V3<R> sv = sc - contact;
    R dist = length(sv);
    R pen = radius / length(sv) - R(1);
    V3<R> pv = mk<R>(pen * sv.x, pen * sv.y, pen * sv.z);
    R plen = length(pv);
    V3<R> pn = normalize(pv);
    R sq = bary.x * bary.x + bary.y * bary.y + bary.z * bary.z;
    if (sq < R(kFloatEpsilon)) return false;
    V3<R> resp = pn * (plen / sq) * ks;
    if (dist > radius) return false;
    out[0] = resp * bary.x; out[1] = resp * bary.y; out[2] = resp * bary.z;
    return true;
}

// collideLaparoscopeDO (integrator.py:981-1050).  The reference subtracts the responses
// from predictedVertex with atomics while other threads read it; here every triangle
// reads the positions as they were when the launch began, and the responses are summed
// per vertex (triangle order) and subtracted afterwards.
template <class R> void collide_all(Sim<R>& s, int64_t f0, int64_t f1) {
    const ffsrl_model* m = s.m;
    R ks = R(s.p->ks_contact);
    for (int64_t f = f0; f < f1; ++f) {
        int env = m->tri_to_env[f];
        if (m->hole[f] == 1) continue;
        int a = m->triangle[3 * f], b = m->triangle[3 * f + 1], c = m->triangle[3 * f + 2];
        V3<R> pA = ld3<R>(s.xp.data(), a), pB = ld3<R>(s.xp.data(), b), pC = ld3<R>(s.xp.data(), c);
        V3<R> centre = (pA + pB + pC) * R(0.3333);
        V3<R> n = normalize(cross(pB - pA, pC - pA));
        V3<R> tA = mk<R>(0, 0, 0), tB = tA, tC = tA;
        R tl = R(0);
        for (int i = 0; i < 3; ++i) {
            int64_t k = int64_t(env) * 4 + i;
            V3<R> base = ld3<R>(m->laparoscope_base, k), tip = ld3<R>(m->laparoscope_tip, k);
            R rad = R(m->laparoscope_radius[k]);
            V3<R> r[3] = {mk<R>(0, 0, 0), mk<R>(0, 0, 0), mk<R>(0, 0, 0)};
            capsule_response(tip, base, rad, n, centre, pA, pB, pC, ks, r);
            tA = tA + r[0]; tB = tB + r[1]; tC = tC + r[2];
            tl = tl + length(r[0]) + length(r[1]) + length(r[2]);
        }
        if (tl > R(0)) s.incol[env] += 1;
        auto add = [&](int vi, V3<R> dv) { s.cdp[3 * vi] += dv.x; s.cdp[3 * vi + 1] += dv.y; s.cdp[3 * vi + 2] += dv.z; };
        if (m->inverse_mass[a] > 0.0f) add(a, tA);
        if (m->inverse_mass[b] > 0.0f) add(b, tB);
        if (m->inverse_mass[c] > 0.0f) add(c, tC);
    }
}

template <class R> void collide_apply(Sim<R>& s, int64_t i) {
    V3<R> x = ld3<R>(s.xp.data(), i);
    V3<R> d = ld3<R>(s.cdp.data(), i);
    st3(s.xp.data(), i, x - d);
    s.cdp[3 * i] = s.cdp[3 * i + 1] = s.cdp[3 * i + 2] = R(0);
}

// bounds (integrator.py:12-21) and PBDStep (integrator.py:23-38)
template <class R> void k_bounds_pbd(Sim<R>& s, int64_t i) {
    R ground = R(s.p->ground_level);
    if (s.xp[3 * i + 1] < ground) s.xp[3 * i + 1] = ground;
    V3<R> x = ld3<R>(s.x.data(), i);
    V3<R> xp = ld3<R>(s.xp.data(), i);
    V3<R> v = (xp - x) * (R(1) / s.dt);
    st3(s.x.data(), i, xp);
    st3(s.v.data(), i, v);
}

struct Range { int64_t v0, v1, t0, t1, e0, e1, f0, f1; };

// one SimIntegratorDO.stepModel over the element ranges in r (integrator.py:1640-1741)
template <class R> void step_range(Sim<R>& s, const Range& r) {
    const ffsrl_params* p = s.p;
    const ffsrl_model* m = s.m;
    uint32_t fl = p->flags;
    R adist = R((double)p->distance_compliance / ((double)p->dt * (double)p->dt));
    R avol = R((double)p->volume_compliance_xpbd / ((double)p->dt * (double)p->dt));
    for (int sub = 0; sub < p->substeps; ++sub) {
        for (int64_t i = r.v0; i < r.v1; ++i) k_gravity(s, i);
        if (fl & FFSRL_DISTANCE_XPBD) for (int64_t e = r.e0; e < r.e1; ++e) s.elam[e] = R(0);
        if (fl & FFSRL_VOLUME_XPBD) for (int64_t t = r.t0; t < r.t1; ++t) s.tlam[t] = R(0);
        for (int it = 0; it < p->iterations; ++it) {
            if (fl & FFSRL_VOLUME) for (int64_t t = r.t0; t < r.t1; ++t) k_volume(s, t);
            if (fl & FFSRL_VOLUME_XPBD) for (int64_t t = r.t0; t < r.t1; ++t) k_volume_xpbd(s, t, avol);
            if (fl & FFSRL_NEOHOOKEAN) for (int64_t t = r.t0; t < r.t1; ++t) k_neohookean(s, t);
            if (fl & FFSRL_DISTANCE) for (int64_t e = r.e0; e < r.e1; ++e) k_distance(s, e);
            if (fl & FFSRL_DISTANCE_XPBD) for (int64_t e = r.e0; e < r.e1; ++e) k_distance_xpbd(s, e, adist);
            for (int64_t i = r.v0; i < r.v1; ++i) k_apply(s, i);
            if (fl & FFSRL_DRAG) for (int64_t i = r.v0; i < r.v1; ++i) k_drag(s, i);
            if ((fl & FFSRL_CONNECTORS) && m->num_connectors > 0)
                for (int64_t c = 0; c < m->num_connectors; ++c) k_connector(s, c);
            if (fl & FFSRL_COLLIDE) {
                collide_all(s, r.f0, r.f1);
                for (int64_t i = r.v0; i < r.v1; ++i) collide_apply(s, i);
            }
        }
        for (int64_t i = r.v0; i < r.v1; ++i) k_bounds_pbd(s, i);
    }
}

template <class R> int run_steps(const ffsrl_model* m, const ffsrl_params* p, int nsteps, int threads,
                                 R* x, R* xp, R* v) {
    Sim<R> s;
    s.m = m; s.p = p;
    int64_t V = m->num_vertices;
    s.x.assign(x, x + 3 * V);
    s.xp.assign(xp, xp + 3 * V);
    s.v.assign(v, v + 3 * V);
    s.dp.assign(3 * V, R(0));
    s.cdp.assign(3 * V, R(0));
    s.cnt.assign(V, 0);
    s.tlam.assign(std::max<int64_t>(m->num_tetrahedrons, 1), R(0));
    s.elam.assign(std::max<int64_t>(m->num_edges, 1), R(0));
    s.incol.assign(std::max(m->num_envs, 1), 0);
    s.dt = R(p->dt);
    // the reference keeps dP and constraintsNumber in the model between launches
    if (m->dp) for (int64_t i = 0; i < 3 * V; ++i) s.dp[i] = R(m->dp[i]);
    if (m->constraints_number) for (int64_t i = 0; i < V; ++i) s.cnt[i] = m->constraints_number[i];

    bool envpar = threads > 1 && m->env_vertex_start && m->env_tet_start && m->env_edge_start && m->env_tri_start &&
                  !((p->flags & FFSRL_CONNECTORS) && m->num_connectors > 0);
    for (int st = 0; st < nsteps; ++st) {
        if (!envpar) {
            Range r{0, V, 0, m->num_tetrahedrons, 0, m->num_edges, 0, m->num_triangles};
            step_range(s, r);
        } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
            for (int e = 0; e < m->num_envs; ++e) {
                Range r{m->env_vertex_start[e], m->env_vertex_start[e + 1], m->env_tet_start[e], m->env_tet_start[e + 1],
                        m->env_edge_start[e], m->env_edge_start[e + 1], m->env_tri_start[e], m->env_tri_start[e + 1]};
                step_range(s, r);
            }
        }
    }
    std::copy(s.x.begin(), s.x.end(), x);
    std::copy(s.xp.begin(), s.xp.end(), xp);
    std::copy(s.v.begin(), s.v.end(), v);
    if (m->dp) for (int64_t i = 0; i < 3 * V; ++i) m->dp[i] = float(s.dp[i]);
    if (m->constraints_number) for (int64_t i = 0; i < V; ++i) m->constraints_number[i] = s.cnt[i];
    if (m->laparoscope_in_collision)
        for (int e = 0; e < m->num_envs; ++e) m->laparoscope_in_collision[e] += s.incol[e];
    if (m->tetrahedron_lambda) for (int64_t t = 0; t < m->num_tetrahedrons; ++t) m->tetrahedron_lambda[t] = float(s.tlam[t]);
    if (m->edge_lambda) for (int64_t e = 0; e < m->num_edges; ++e) m->edge_lambda[e] = float(s.elam[e]);
    return 0;
}

// ---------------------------------------------------------------------------------
// BVH refit (bvh.py:30-104), all levels deepest first.
void refit_node_level(const ffsrl_bvh* b, const float* pts, const int32_t* faces, int e, int L);

void refit(const ffsrl_bvh* b, const float* pts, const int32_t* faces) {
    for (int L = b->max_level; L >= 0; --L)
        for (int e = 0; e < b->num_envs; ++e) refit_node_level(b, pts, faces, e, L);
}

// refitBVHLevel's face shift (bvh.py:66-74).  The reference orders visual faces object by
// object over all envs -- [mesh faces of every env][rigid faces of every env][instrument
// faces of every env], M, Rg and Lf faces per env -- and its refit maps env e's local face
// t with `>` where the traversal (render.py:462-470) uses `>=`, so local faces M and M + Rg
// are boxed from another env's face.  Written here as the env-major global face id the
// refit reads for each (env, local face): out[env_face_offset[e] + t].
extern "C" void oracle_reference_refit_source(int N, int M, int Rg, int Lf, const int32_t* env_face_offset,
                                              int32_t* out) {
    const int F = M + Rg + Lf;
    for (int e = 0; e < N; ++e)
        for (int t = 0; t < F; ++t) {
            int64_t g;
            if (t > M + Rg) g = t + int64_t(N - 1) * (M + Rg) + int64_t(e) * Lf;
            else if (t > M) g = t + int64_t(N - 1) * M + int64_t(e) * Rg;
            else g = t + int64_t(e) * M;
            int64_t env, loc;
            if (g < int64_t(N) * M) {
                env = g / M; loc = g % M;
            } else if (g < int64_t(N) * (M + Rg)) {
                int64_t h = g - int64_t(N) * M;
                env = h / Rg; loc = M + h % Rg;
            } else {
                int64_t h = g - int64_t(N) * (M + Rg);
                env = h / Lf; loc = M + Rg + h % Lf;
            }
            out[env_face_offset[e] + t] = int32_t(env_face_offset[env] + loc);
        }
}

// one env's tree, all levels deepest first
void refit_env(const ffsrl_bvh* b, const float* pts, const int32_t* faces, int e) {
    for (int L = b->max_level; L >= 0; --L) refit_node_level(b, pts, faces, e, L);
}

// the nodes of env e at level L
void refit_node_level(const ffsrl_bvh* b, const float* pts, const int32_t* faces, int e, int L) {
    int topo = b->env_topology[e];
    int n0 = b->topo_node_offset[topo], n1 = b->topo_node_offset[topo + 1];
    int t0 = b->topo_tri_offset[topo];
    int base = b->env_node_offset[e];
    for (int n = 0; n < n1 - n0; ++n) {
        if (b->level[n0 + n] != L) continue;
        int left = b->left_node[n0 + n];
        V3<float> lo, hi;
        if (left < 0) {
            lo = mk<float>(1e6f, 1e6f, 1e6f);
            hi = mk<float>(-1e6f, -1e6f, -1e6f);
            int first = b->first_tri_id[n0 + n];
            for (int k = 0; k < b->tri_count[n0 + n]; ++k) {
                int64_t f = int64_t(b->env_face_offset[e]) + b->tri_id[t0 + first + k];
                if (b->refit_source) f = b->refit_source[f];  // the face the reference's refit boxes
                V3<float> pA = ld3<float>(pts, faces[3 * f]), pB = ld3<float>(pts, faces[3 * f + 1]),
                          pC = ld3<float>(pts, faces[3 * f + 2]);
                lo = vmin(pA, vmin(pB, vmin(pC, lo)));
                hi = vmax(pA, vmax(pB, vmax(pC, hi)));
            }
        } else {
            V3<float> l0 = ld3<float>(b->aabb_min, base + left), h0 = ld3<float>(b->aabb_max, base + left);
            V3<float> l1 = ld3<float>(b->aabb_min, base + left + 1), h1 = ld3<float>(b->aabb_max, base + left + 1);
            lo = vmin(l0, l1);
            hi = vmax(h0, h1);
        }
        st3(b->aabb_min, base + n, lo);
        st3(b->aabb_max, base + n, hi);
    }
}

// ---------------------------------------------------------------------------------
// Renderer (render.py:81-121, 276-498, 588-697, 699-724), vertex-colour and depth.
inline V3<float> quat_rotate(const float* q, V3<float> x) {
    V3<float> u = mk<float>(q[0], q[1], q[2]);
    float w = q[3];
    float c = 2.0f * w * w - 1.0f;
    float d = 2.0f * (u.x * x.x + u.y * x.y + u.z * x.z);
    return x * c + u * d + cross(u, x) * (w * 2.0f);
}

struct Hit { int tri; float t; V3<float> p; };

// index of the object of env e holding env-local face lf (visFaceToObjectId, render.py:360):
// the last of the env's objects whose first face is <= lf
int object_of(const ffsrl_render* r, int e, int lf) {
    int o0 = r->env_objects[2 * e], no = r->env_objects[2 * e + 1];
    int k = 0;
    while (k + 1 < no && r->object_texture[5 * (o0 + k + 1)] <= lf) ++k;
    return o0 + k;
}

// intersectAABB (render.py:588-609): returns hit flag and tmin
inline bool slab(V3<float> ro, V3<float> rd, V3<float> lo, V3<float> hi, float* tnear) {
    float t1 = (lo.x - ro.x) / rd.x, t2 = (hi.x - ro.x) / rd.x;
    float t3 = (lo.y - ro.y) / rd.y, t4 = (hi.y - ro.y) / rd.y;
    float t5 = (lo.z - ro.z) / rd.z, t6 = (hi.z - ro.z) / rd.z;
    float tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
    float tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
    if ((tmax >= 0.0f) && (tmax >= tmin)) { *tnear = tmin; return true; }
    *tnear = 0.0f;
    return false;
}

// MTTriRayIntersection (render.py:661-697): t (or -1) and the hit point
inline float moller_trumbore(V3<float> a, V3<float> b, V3<float> c, V3<float> ro, V3<float> rd, V3<float>* p) {
    V3<float> ab = b - a, ac = c - a;
    V3<float> pvec = cross(rd, ac);
    float det = dot(ab, pvec);
    if (std::fabs(det) < 0.0001f) return -1.0f;
    float invDet = 1.0f / det;
    V3<float> tvec = ro - a;
    float u = dot(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    V3<float> qvec = cross(tvec, ab);
    float v = dot(rd, qvec) * invDet;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    float t = dot(ac, qvec) * invDet;
    *p = ro + t * rd;
    return t;
}

// meshQueryRayManyEnvs (render.py:411-498) with a stack of `cap` entries
int query(const ffsrl_bvh* b, const ffsrl_render* r, int e, V3<float> ro, V3<float> rd, Hit* h, int cap) {
    int topo = b->env_topology[e];
    int n0 = b->topo_node_offset[topo];
    int nn = b->topo_node_offset[topo + 1] - n0;
    int t0 = b->topo_tri_offset[topo];
    int base = b->env_node_offset[e];
    int64_t fofs = b->env_face_offset[e];
    int visits = 0;
    int stack[256];
    int count = 1;
    stack[0] = 0;
    float tMin = 1e6f;
    const float tMax = 1e6f;
    h->tri = -1; h->t = 0.0f; h->p = mk<float>(0, 0, 0);
    while (count) {
        int node = stack[--count];
        if (++visits > nn) return FFSRL_ERR_STACK_OVERFLOW;  // a valid tree visits each node once
        V3<float> lo = ld3<float>(b->aabb_min, base + node), hi = ld3<float>(b->aabb_max, base + node);
        float tn;
        bool hit = slab(ro, rd, lo, hi, &tn);
        if (hit && tn < tMin) {
            int left = b->left_node[n0 + node];
            if (left == -1) {
                int first = b->first_tri_id[n0 + node];
                for (int k = 0; k < b->tri_count[n0 + node]; ++k) {
                    int64_t f = fofs + b->tri_id[t0 + first + k];
                    V3<float> A = ld3<float>(r->vis_point, r->vis_face[3 * f]);
                    V3<float> B = ld3<float>(r->vis_point, r->vis_face[3 * f + 1]);
                    V3<float> C = ld3<float>(r->vis_point, r->vis_face[3 * f + 2]);
                    V3<float> p;
                    float t = moller_trumbore(A, B, C, ro, rd, &p);
                    if (t < tMin && t > 0.0f) {
                        tMin = t;
                        h->tri = int(f); h->t = t; h->p = p;
                    }
                }
            } else {
                if (left < 0 || left + 1 >= nn) return FFSRL_ERR_INVALID_ARGUMENT;
                if (count + 2 > cap) return FFSRL_ERR_STACK_OVERFLOW;
                stack[count] = left;
                stack[count + 1] = left + 1;
                count += 2;
            }
        }
    }
    if (tMin >= tMax) { h->tri = -1; h->t = 0.0f; h->p = mk<float>(0, 0, 0); }
    return 0;
}

int render_env(const ffsrl_render* r, const ffsrl_bvh* b, int stack_cap, int e, const float* nrmp,
               std::vector<float>& ray, std::vector<float>& rdep);

// Normals serially in face order, then each env's rays; `threads` > 1 spreads the envs
// over OpenMP threads (envs share nothing, so the images are the same).
int render(const ffsrl_render* r, const ffsrl_bvh* b, int stack_cap, int threads = 1) {
    int64_t P = r->num_vis_points;
    std::vector<float> nsum(3 * P, 0.0f);
    for (int64_t f = 0; f < r->num_vis_faces; ++f) {  // vertex_normal_sum_kernel, serial order
        int i = r->vis_face[3 * f], j = r->vis_face[3 * f + 1], k = r->vis_face[3 * f + 2];
        V3<float> a = ld3<float>(r->vis_point, i), bb = ld3<float>(r->vis_point, j), c = ld3<float>(r->vis_point, k);
        V3<float> an = cross(bb - a, c - a);
        for (int v : {i, j, k}) { nsum[3 * v] += an.x; nsum[3 * v + 1] += an.y; nsum[3 * v + 2] += an.z; }
    }
    std::vector<float> nrm(3 * P);
    for (int64_t i = 0; i < P; ++i) st3(nrm.data(), i, normalize(ld3<float>(nsum.data(), i)));
    if (r->vertex_normal) std::copy(nrm.begin(), nrm.end(), r->vertex_normal);

    const int R = r->resolution, W = 2 * R, H = 2 * R;
    int status = 0;
    if (threads <= 1) {
        std::vector<float> ray(3 * (size_t)W * H), rdep((size_t)W * H);
        for (int e = 0; e < r->num_envs && !status; ++e) status = render_env(r, b, stack_cap, e, nrm.data(), ray, rdep);
        return status;
    }
#pragma omp parallel num_threads(threads)
    {
        std::vector<float> ray(3 * (size_t)W * H), rdep((size_t)W * H);
#pragma omp for schedule(dynamic, 1)
        for (int e = 0; e < r->num_envs; ++e) {
            int st = render_env(r, b, stack_cap, e, nrm.data(), ray, rdep);
            if (st) {
#pragma omp critical
                status = st;
            }
        }
    }
    return status;
}

int render_env(const ffsrl_render* r, const ffsrl_bvh* b, int stack_cap, int e, const float* nrmp,
               std::vector<float>& ray, std::vector<float>& rdep) {
    const int R = r->resolution, W = 2 * R, H = 2 * R;
    {
        int cam = r->num_cameras > 1 ? e : 0;
        V3<float> ro = ld3<float>(r->camera_pos, cam);
        const float* q = r->camera_rot + 4 * cam;
        for (int tid = 0; tid < W * H; ++tid) {  // drawSimBVHKernelManyEnvs (render.py:276-409)
            int x = tid % W;
            int y = H - tid / W;
            float sx = 2.0f * float(x) / float(W) - 1.0f;
            float sy = 2.0f * float(y) / float(H) - 1.0f;
            V3<float> rd = normalize(quat_rotate(q, mk<float>(sx * r->camera_tan * r->camera_aspect, sy * r->camera_tan, -1.0f)));
            Hit h;
            int st = query(b, r, e, ro, rd, &h, stack_cap);
            if (st) return st;
            V3<float> col = mk<float>(0, 0, 0);
            float dep = 0.0f;
            if (h.tri > -1) {
                int i = r->vis_face[3 * (int64_t)h.tri], j = r->vis_face[3 * (int64_t)h.tri + 1], k = r->vis_face[3 * (int64_t)h.tri + 2];
                V3<float> a = ld3<float>(r->vis_point, i), bb = ld3<float>(r->vis_point, j), c = ld3<float>(r->vis_point, k);
                V3<float> p = h.p;
                float area = length(cross(bb - a, c - a));
                float w = length(cross(bb - a, p - a)) / area;
                float v = length(cross(p - a, c - a)) / area;
                float u = 1.0f - w - v;
                V3<float> n = u * ld3<float>(nrmp, i) + v * ld3<float>(nrmp, j) + w * ld3<float>(nrmp, k);
                if (r->render_mode == 2) {  // normal map (render.py:399-401)
                    col = n * 0.5f + mk<float>(0.5f, 0.5f, 0.5f);
                } else if (r->render_mode == 4) {  // depth map (render.py:403-405)
                    float g = h.t / 50.0f;
                    col = mk<float>(g, g, g);
                } else {
                    V3<float> base;
                    if (r->render_mode == 0) {  // grayscale
                        base = mk<float>(1.0f, 1.0f, 1.0f);
                    } else if (r->render_mode == 1 && r->env_objects &&
                               r->object_texture[5 * object_of(r, e, int(h.tri - b->env_face_offset[e])) + 2] > 0) {
                        // texture_interpolation (render.py:123-148), indices clamped into the texture
                        int lf = (int)(h.tri - b->env_face_offset[e]);
                        const int32_t* ob = r->object_texture + 5 * object_of(r, e, lf);
                        int first = ob[1], S = ob[2], c0 = ob[3];
                        const int32_t* ti = r->tex_indices + ob[4] + 3 * (lf - ob[0]);
                        const float* ta = r->tex_coords + 2 * (c0 + ti[0]);
                        const float* tb = r->tex_coords + 2 * (c0 + ti[1]);
                        const float* tc = r->tex_coords + 2 * (c0 + ti[2]);
                        float tx = (u * ta[0] + v * tb[0]) + w * tc[0];
                        float ty = (u * ta[1] + v * tb[1]) + w * tc[1];
                        float fx = tx * float(S - 1), fy = (1.0f - ty) * float(S - 1);
                        int x0 = (int)fx, y0 = (int)fy;
                        float ax = fx - float(x0), ay = fy - float(y0);
                        int x1 = x0 + 1, y1 = y0 + 1;
                        auto cl = [S](int q) { return q < 0 ? 0 : (q > S - 1 ? S - 1 : q); };
                        x0 = cl(x0); x1 = cl(x1); y0 = cl(y0); y1 = cl(y1);
                        V3<float> c00 = ld3<float>(r->texture, (int64_t)first + y0 + x0 * S);
                        V3<float> c10 = ld3<float>(r->texture, (int64_t)first + y0 + x1 * S);
                        V3<float> c01 = ld3<float>(r->texture, (int64_t)first + y1 + x0 * S);
                        V3<float> c11 = ld3<float>(r->texture, (int64_t)first + y1 + x1 * S);
                        V3<float> lower = (1.0f - ax) * c00 + ax * c10;
                        V3<float> upper = (1.0f - ax) * c01 + ax * c11;
                        base = (1.0f - ay) * lower + ay * upper;
                    } else {
                        base = (ld3<float>(r->vis_point_color, i) + ld3<float>(r->vis_point_color, j) +
                                ld3<float>(r->vis_point_color, k)) / 3.0f;
                    }
                    float lam = 0.0f;
                    for (int l = 0; l < r->num_lights; ++l) {
                        V3<float> dir = ld3<float>(r->light_dir, l);
                        float val = r->light_intensity[l] * dot(n, dir);
                        if (val < 0.0f) val = 0.0f;
                        lam = lam + val;
                    }
                    col = lam * base;
                }
                if (col.x > 1.0f) col.x = 1.0f;
                if (col.y > 1.0f) col.y = 1.0f;
                if (col.z > 1.0f) col.z = 1.0f;
                dep = h.t / 50.0f;
                if (dep > 1.0f) dep = 1.0f;
            }
            st3(ray.data(), tid, col);
            rdep[tid] = dep;
        }
        for (int pix = 0; pix < R * R; ++pix) {  // downsample_kernel (render.py:699-724)
            int px = pix % R, py = pix / R;
            int start = py * 2 * W + px * 2;
            V3<float> c = mk<float>(0, 0, 0);
            float d = 0.0f;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    V3<float> s = ld3<float>(ray.data(), start + i * W + j);
                    c = mk<float>(c.x + s.x, c.y + s.y, c.z + s.z);
                    d = d + rdep[start + i * W + j];
                }
            float nsq = float(2 * 2);
            int64_t o = (int64_t)e * R * R + pix;
            if (r->color) st3(r->color, o, mk<float>(c.x / nsq, c.y / nsq, c.z / nsq));
            if (r->depth) r->depth[o] = d / nsq;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------------
// Instrument kinematics (modelDO.py:26-416): 7 transforms per env stored as the
// reference stores them (row-major transpose of the column-vector transform); children
// follow their parent: 0 -> 1 2 4 5 6, 3 -> 0 1 2 4 5 6, 4 -> 1, 5 -> 2.  Per env the rod,
// rotation-centre and clamp actions apply in that order.  Warp's mat44(pos, quat, scale),
// inverse and quat_from_axis_angle are restated from their mathematics.
struct Mat4 { float m[4][4]; };
struct P3 { float x, y, z; };
inline P3 p3(float x, float y, float z) { return P3{x, y, z}; }
inline float pdot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float plen(P3 a) { return std::sqrt(pdot(a, a)); }

Mat4 kload(const float* X, int s) {
    Mat4 c;
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) c.m[r][k] = X[16 * s + 4 * k + r];
    return c;
}
void kstore(float* X, int s, const Mat4& c) {
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) X[16 * s + 4 * k + r] = c.m[r][k];
}
Mat4 kmul(const Mat4& a, const Mat4& b) {
    Mat4 c;
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k)
            c.m[r][k] = ((a.m[r][0] * b.m[0][k] + a.m[r][1] * b.m[1][k]) + a.m[r][2] * b.m[2][k]) + a.m[r][3] * b.m[3][k];
    return c;
}
// adjugate / determinant with the 2x2 minors of the row pairs (0,1) and (2,3)
Mat4 kinv(const Mat4& a) {
    const float(*m)[4] = a.m;
    float s0 = m[0][0] * m[1][1] - m[1][0] * m[0][1], s1 = m[0][0] * m[1][2] - m[1][0] * m[0][2];
    float s2 = m[0][0] * m[1][3] - m[1][0] * m[0][3], s3 = m[0][1] * m[1][2] - m[1][1] * m[0][2];
    float s4 = m[0][1] * m[1][3] - m[1][1] * m[0][3], s5 = m[0][2] * m[1][3] - m[1][2] * m[0][3];
    float c5 = m[2][2] * m[3][3] - m[3][2] * m[2][3], c4 = m[2][1] * m[3][3] - m[3][1] * m[2][3];
    float c3 = m[2][1] * m[3][2] - m[3][1] * m[2][2], c2 = m[2][0] * m[3][3] - m[3][0] * m[2][3];
    float c1 = m[2][0] * m[3][2] - m[3][0] * m[2][2], c0 = m[2][0] * m[3][1] - m[3][0] * m[2][1];
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    float inv = 1.0f / det;
    Mat4 b;
    b.m[0][0] = (m[1][1] * c5 - m[1][2] * c4 + m[1][3] * c3) * inv;
    b.m[0][1] = (-m[0][1] * c5 + m[0][2] * c4 - m[0][3] * c3) * inv;
    b.m[0][2] = (m[3][1] * s5 - m[3][2] * s4 + m[3][3] * s3) * inv;
    b.m[0][3] = (-m[2][1] * s5 + m[2][2] * s4 - m[2][3] * s3) * inv;
    b.m[1][0] = (-m[1][0] * c5 + m[1][2] * c2 - m[1][3] * c1) * inv;
    b.m[1][1] = (m[0][0] * c5 - m[0][2] * c2 + m[0][3] * c1) * inv;
    b.m[1][2] = (-m[3][0] * s5 + m[3][2] * s2 - m[3][3] * s1) * inv;
    b.m[1][3] = (m[2][0] * s5 - m[2][2] * s2 + m[2][3] * s1) * inv;
    b.m[2][0] = (m[1][0] * c4 - m[1][1] * c2 + m[1][3] * c0) * inv;
    b.m[2][1] = (-m[0][0] * c4 + m[0][1] * c2 - m[0][3] * c0) * inv;
    b.m[2][2] = (m[3][0] * s4 - m[3][1] * s2 + m[3][3] * s0) * inv;
    b.m[2][3] = (-m[2][0] * s4 + m[2][1] * s2 - m[2][3] * s0) * inv;
    b.m[3][0] = (-m[1][0] * c3 + m[1][1] * c1 - m[1][2] * c0) * inv;
    b.m[3][1] = (m[0][0] * c3 - m[0][1] * c1 + m[0][2] * c0) * inv;
    b.m[3][2] = (-m[3][0] * s3 + m[3][1] * s1 - m[3][2] * s0) * inv;
    b.m[3][3] = (m[2][0] * s3 - m[2][1] * s1 + m[2][2] * s0) * inv;
    return b;
}
P3 kpoint(const Mat4& c, P3 p) {
    return p3(((c.m[0][0] * p.x + c.m[0][1] * p.y) + c.m[0][2] * p.z) + c.m[0][3],
              ((c.m[1][0] * p.x + c.m[1][1] * p.y) + c.m[1][2] * p.z) + c.m[1][3],
              ((c.m[2][0] * p.x + c.m[2][1] * p.y) + c.m[2][2] * p.z) + c.m[2][3]);
}
// wp.mat44(t, quat_from_axis_angle(axis, angle), 1)
Mat4 krigid(P3 t, P3 axis, float angle) {
    float h = 0.5f * angle;
    float s = std::sin(h), w = std::cos(h);
    float x = axis.x * s, y = axis.y * s, z = axis.z * s;
    Mat4 c;
    c.m[0][0] = 1.0f - 2.0f * (y * y + z * z); c.m[0][1] = 2.0f * (x * y - z * w); c.m[0][2] = 2.0f * (x * z + y * w);
    c.m[1][0] = 2.0f * (x * y + z * w); c.m[1][1] = 1.0f - 2.0f * (x * x + z * z); c.m[1][2] = 2.0f * (y * z - x * w);
    c.m[2][0] = 2.0f * (x * z - y * w); c.m[2][1] = 2.0f * (y * z + x * w); c.m[2][2] = 1.0f - 2.0f * (x * x + y * y);
    c.m[0][3] = t.x; c.m[1][3] = t.y; c.m[2][3] = t.z;
    c.m[3][0] = 0.0f; c.m[3][1] = 0.0f; c.m[3][2] = 0.0f; c.m[3][3] = 1.0f;
    return c;
}
// getTransformationMatrix (modelDO.py:396-414)
Mat4 kshift_rotate(float sx, float sy, float sz, float ax, float ay, float az) {
    const P3 zero = p3(0.0f, 0.0f, 0.0f);
    Mat4 T = krigid(p3(sx, sy, sz), zero, 0.0f);
    Mat4 X = krigid(zero, p3(1.0f, 0.0f, 0.0f), ax);
    Mat4 Y = krigid(zero, p3(0.0f, 1.0f, 0.0f), ay);
    Mat4 Z = krigid(zero, p3(0.0f, 0.0f, 1.0f), az);
    return kmul(T, kmul(X, kmul(Y, Z)));
}
// applyTransformationToChild (modelDO.py:386-394)
void kchild(float* X, const Mat4& M, int parent, int child) {
    Mat4 P = kload(X, parent);
    Mat4 C = kload(X, child);
    kstore(X, child, kmul(P, kmul(M, kmul(kinv(P), C))));
}
// applyTransformationToChildren (modelDO.py:366-384)
void kchildren(float* X, const Mat4& M, int parent) {
    if (parent == 4) kchild(X, M, 4, 1);
    if (parent == 5) kchild(X, M, 5, 2);
    if (parent == 3)
        for (int i = 0; i < 7; ++i)
            if (i != 3) kchild(X, M, 3, i);
    if (parent == 0)
        for (int i = 1; i < 7; ++i)
            if (i != 3) kchild(X, M, 0, i);
}
// transformFunc (modelDO.py:291-298)
void kslot(float* X, int slot, const Mat4& cur, const Mat4& M) {
    kchildren(X, M, slot);
    kstore(X, slot, kmul(cur, M));
}
// rotateClampsFunc (modelDO.py:300-364), angles in degrees
void kclamps(float* X, int* dch, int* dchu, float action) {
    const float pi = 3.14159265358979323846f;
    float diff = action * 180.0f / pi;
    if (diff == 0.0f) return;
    Mat4 rod = kload(X, 0), left = kload(X, 4), right = kload(X, 5);
    Mat4 local = kmul(kinv(rod), right);
    float cur = std::asin(local.m[2][1]) * 180.0f / pi;
    bool apply = false;
    if (dch[0] == 1 && dchu[0] == 1) dchu[0] = 0;
    if (action > 0.0f) {
        if (cur < 85.0f) {
            if (cur + diff > 85.0f) diff = 85.0f - cur;
            apply = true;
        }
        if (cur > 3.0f + 40.0f && dch[0] == 1) { dch[0] = 0; dchu[0] = 1; }
    } else {
        if (cur > 40.0f) {
            if (cur + diff < 40.0f) diff = 40.0f - cur;
            apply = true;
        }
        if (cur < 3.0f + 40.0f && dch[0] == 0) { dch[0] = 1; dchu[0] = 1; }
    }
    if (apply) {
        float rad = diff * pi / 180.0f;
        Mat4 R = kshift_rotate(0.0f, 0.0f, 0.0f, rad, 0.0f, 0.0f);
        Mat4 Ri = kshift_rotate(0.0f, 0.0f, 0.0f, -rad, 0.0f, 0.0f);
        kstore(X, 4, kmul(left, Ri));
        kchildren(X, Ri, 4);
        kstore(X, 5, kmul(right, R));
        kchildren(X, R, 5);
    }
}
// updateLaparoscopeKernel (modelDO.py:222-245)
void kends(const float* X, const float* height, float* base, float* tip, int e) {
    for (int k = 0; k < 4; ++k) {
        Mat4 c;
        P3 bl, tl;
        if (k < 3) {
            c = kload(X, k);
            float h = height[4 * e + k];
            bl = p3(0.0f, 0.0f, 0.0f - h / 1.85f);
            tl = p3(0.0f, 0.0f, 0.0f + h / 1.85f);
        } else {
            c = kload(X, 0);
            float rh = height[4 * e], ch = height[4 * e + 2];
            bl = p3(0.0f, 0.0f, 0.0f - rh * 0.5f - ch * 1.0f);
            tl = p3(0.0f, 0.0f, 0.0f + rh * 0.5f + ch * 1.0f);
        }
        P3 b = kpoint(c, bl), t = kpoint(c, tl);
        int64_t o = 3ll * (4 * e + k);
        base[o] = b.x; base[o + 1] = b.y; base[o + 2] = b.z;
        tip[o] = t.x; tip[o + 1] = t.y; tip[o + 2] = t.z;
    }
}

}  // namespace

extern "C" {

int oracle_step_f32(const ffsrl_model* m, const ffsrl_params* p, int nsteps, int threads) {
    return run_steps<float>(m, p, nsteps, threads, m->vertex, m->predicted_vertex, m->velocity);
}

// FP64 run of the same kernels: state arrays are double [3V]; constants are the float
// arrays of m promoted on read.
int oracle_step_f64(const ffsrl_model* m, const ffsrl_params* p, int nsteps, int threads, double* x, double* xp,
                    double* v) {
    return run_steps<double>(m, p, nsteps, threads, x, xp, v);
}

void oracle_remap(float* dst, const float* src, const int32_t* map, int32_t count) {
    for (int i = 0; i < count; ++i) {  // remapAToBKernel (utils.py:32-42)
        int a = map[2 * i], b = map[2 * i + 1];
        dst[3 * a] = src[3 * b]; dst[3 * a + 1] = src[3 * b + 1]; dst[3 * a + 2] = src[3 * b + 2];
    }
}

void oracle_refit(const ffsrl_bvh* b, const float* pts, const int32_t* faces) { refit(b, pts, faces); }

int oracle_render(const ffsrl_render* r, const ffsrl_bvh* b, int stack_cap) { return render(r, b, stack_cap); }

// Same images as oracle_render, envs spread over `threads` host threads (CPU timing).
int oracle_render_mt(const ffsrl_render* r, const ffsrl_bvh* b, int stack_cap, int threads) {
    return render(r, b, stack_cap, threads);
}

// Same boxes as oracle_refit, envs spread over `threads` host threads: each env's tree
// is refit bottom-up on its own (the levels of one env stay in order).
void oracle_refit_mt(const ffsrl_bvh* b, const float* pts, const int32_t* faces, int threads) {
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int e = 0; e < b->num_envs; ++e) refit_env(b, pts, faces, e);
}


// Instrument kinematics entry points (host arrays; same layouts as the library's)
void oracle_instrument_update(const float* xform, float* base, float* tip, const float* height, int num_envs) {
    for (int e = 0; e < num_envs; ++e) kends(xform + 112ll * e, height, base, tip, e);
}

void oracle_instrument_apply_actions(float* xform, const float* actions, int* dch, int* dchu, float* base, float* tip,
                                     const float* height, int num_envs) {
    for (int e = 0; e < num_envs; ++e) {  // applyActionsKernel (modelDO.py:161-190)
        float* X = xform + 112ll * e;
        const float* a = actions + 5ll * e;
        Mat4 rod0 = kload(X, 0), rc0 = kload(X, 3);
        kslot(X, 0, rod0, kshift_rotate(0.0f, 0.0f, a[0], 0.0f, 0.0f, a[1]));
        kslot(X, 3, rc0, kshift_rotate(0.0f, 0.0f, 0.0f, a[2], a[3], 0.0f));
        kclamps(X, dch + 3ll * e, dchu + 3ll * e, a[4]);
        kends(X, height, base, tip, e);
    }
}

void oracle_instrument_cartesian(float* xform, const float* actions, const float* ws, int* violation, float* base,
                                 float* tip, const float* height, int num_envs) {
    for (int e = 0; e < num_envs; ++e) {  // transfromCartesianActionsKernel[InWorkspace] (modelDO.py:56-153)
        const float* a = actions + 3ll * e;
        if (a[0] == 0.0f && a[1] == 0.0f && a[2] == 0.0f) continue;
        float* X = xform + 112ll * e;
        int64_t d = 3ll * (4 * e + 3);
        P3 cur = p3(tip[d], tip[d + 1], tip[d + 2]);
        P3 act = p3(a[0], a[1], a[2]);
        if (ws) {
            if (violation) violation[e] = 0;
            P3 nw = p3(cur.x + act.x, cur.y + act.y, cur.z + act.z);
            if (nw.x < ws[0] || nw.x > ws[3]) { act.x = 0.0f; if (violation) violation[e] = 1; }
            if (nw.y < ws[1] || nw.y > ws[4]) { act.y = 0.0f; if (violation) violation[e] = 1; }
            if (nw.z < ws[2] || nw.z > ws[5]) { act.z = 0.0f; if (violation) violation[e] = 1; }
        }
        Mat4 rod = kload(X, 0), rc = kload(X, 3);
        P3 rel = kpoint(kinv(rc), cur);
        P3 delta = p3(((rc.m[0][0] * act.x + rc.m[1][0] * act.y) + rc.m[2][0] * act.z) + rc.m[3][0],
                      ((rc.m[0][1] * act.x + rc.m[1][1] * act.y) + rc.m[2][1] * act.z) + rc.m[3][1],
                      ((rc.m[0][2] * act.x + rc.m[1][2] * act.y) + rc.m[2][2] * act.z) + rc.m[3][2]);
        P3 nrel = p3(rel.x + delta.x, rel.y + delta.y, rel.z + delta.z);
        float rcur = plen(rel), rnew = plen(nrel);
        P3 cr = p3(rel.y * nrel.z - rel.z * nrel.y, rel.z * nrel.x - rel.x * nrel.z, rel.x * nrel.y - rel.y * nrel.x);
        float sin_t = plen(cr) / (plen(rel) * plen(nrel));
        float lc = plen(cr);
        P3 axis = lc > 0.0f ? p3(cr.x / lc, cr.y / lc, cr.z / lc) : p3(0.0f, 0.0f, 0.0f);
        float angle = std::asin(sin_t);
        kslot(X, 0, rod, kshift_rotate(0.0f, 0.0f, rnew - rcur, 0.0f, 0.0f, 0.0f));
        kslot(X, 3, rc, krigid(p3(0.0f, 0.0f, 0.0f), axis, angle));
        kends(X, height, base, tip, e);
    }
}

void oracle_instrument_set_rotation_center(float* xform, const float* t, const float* r, float* base, float* tip,
                                           const float* height, int num_envs) {
    for (int e = 0; e < num_envs; ++e) {  // setRotationCenterTransformKernel (modelDO.py:155-171)
        float* X = xform + 112ll * e;
        Mat4 rc = kload(X, 3);
        int64_t o = 3ll * e;
        Mat4 G = kshift_rotate(t[o], t[o + 1], t[o + 2], r[o], r[o + 1], r[o + 2]);
        kslot(X, 3, rc, kmul(kinv(rc), G));
        kends(X, height, base, tip, e);
    }
}

// updateLaparoscopeMeshKernel (modelDO.py:202-216) over every env, as
// transformSimLaparoscopeMeshData launches it (modelDO.py:1446-1473): the env's transform of
// the point's slot, transposed out of storage, applied to the shared local point
void oracle_instrument_visual(const float* xform, const float* local, const int* slot, int num_points, float* vis,
                              const int* env_first_point, int num_envs) {
    for (int e = 0; e < num_envs; ++e) {
        const float* X = xform + 112ll * e;
        for (int i = 0; i < num_points; ++i) {
            if (slot[i] < 0 || slot[i] > 6) continue;
            P3 p = kpoint(kload(X, slot[i]), p3(local[3 * i], local[3 * i + 1], local[3 * i + 2]));
            int64_t o = 3ll * ((int64_t)env_first_point[e] + i);
            vis[o] = p.x; vis[o + 1] = p.y; vis[o + 2] = p.z;
        }
    }
}

// ---- cutting and heating (integrator.py:700-918, 1153-1185, 1406-1518, 1583-1605),
// serial in thread order.  Map entries of -1 are skipped (the reference would index with
// them).  An element's env comes from the optional env map (env 0 without it, the
// reference's single instrument); a tet scan for an edge visits every tet, as the
// reference does.

// edgeBreakerKernel (integrator.py:700-731)
void oracle_edge_breaker(const float* xp, const int* edge, const float* rest, const float* active, float* value,
                         int ne, float factor, float threshold) {
    for (int t = 0; t < ne; ++t) {
        if (active[t] == 0.0f) continue;
        float L0 = rest[t];
        if (L0 < float(kFloatEpsilon)) continue;
        float len = length(ld3<float>(xp, edge[2 * t + 1]) - ld3<float>(xp, edge[2 * t]));
        if (len < float(kFloatEpsilon)) continue;
        float C = len / L0 - 1.0f;
        if (C > threshold) value[t] = value[t] + (C - threshold) * factor;
    }
}

static bool tet_holds(const int* q, int v) { return v == q[0] || v == q[1] || v == q[2] || v == q[3]; }

// checkEdgeBreakerKernel (integrator.py:733-775); the tet flag indexed by the edge id is
// the reference's, applied only where that id is a tet id
void oracle_check_edge_breaker(const float* value, const int* edge, const float* active_edge, int* flip_edges, int ne,
                               const int* tet, int nt, const float* active_tet, int* flip_tets, const int* edge_tris,
                               int* holes, float limit) {
    for (int t = 0; t < ne; ++t) {
        if (!(value[t] > limit)) continue;
        if (flip_edges[t] == 0 && active_edge[t] == 1.0f) flip_edges[t] = -1;
        int a = edge[2 * t], b = edge[2 * t + 1];
        for (int k = 0; k < 2; ++k)
            if (edge_tris[2 * t + k] > -1) holes[edge_tris[2 * t + k]] = 1;
        if (t >= nt) continue;
        for (int i = 0; i < nt; ++i)
            if (tet_holds(tet + 4 * i, a) && tet_holds(tet + 4 * i, b) && flip_tets[t] == 0 && active_tet[t] == 1.0f)
                flip_tets[t] = -1;
    }
}

// tetrahedronBreaker (integrator.py:777-818)
void oracle_tetrahedron_breaker(const float* xp, const int* tet, const float* rest, const float* active, float* value,
                                int nt, float factor) {
    for (int t = 0; t < nt; ++t) {
        if (!(active[t] == 1.0f)) continue;
        V3<float> pa = ld3<float>(xp, tet[4 * t]);
        V3<float> p1 = ld3<float>(xp, tet[4 * t + 1]) - pa, p2 = ld3<float>(xp, tet[4 * t + 2]) - pa,
                  p3 = ld3<float>(xp, tet[4 * t + 3]) - pa;
        float C = dot(cross(p1, p2), p3) / 6.0f - rest[t];
        if (C > 0.0f) value[t] = value[t] + C * factor;
    }
}

// tetrahedronHeatPropagation (integrator.py:820-847)
void oracle_heat_propagation(const float* active, const int* nbr, const float* heat, float* new_heat, int nt,
                             float conduction, float transfer, float loss) {
    for (int t = 0; t < nt; ++t) {
        if (active[t] == 0.0f) continue;
        float h = heat[t], avg = 0.0f;
        for (int i = 0; i < 4; ++i) {
            int n = nbr[4 * t + i];
            if (n > -1 && active[n] > 0.0f) avg = avg + (heat[n] - h) * conduction;
        }
        new_heat[t] = h * (1.0f - loss) + avg * transfer;
    }
}

// tetrahedronHeatUpdate (integrator.py:849-872): a vertex keeps the last write, the
// highest tet id holding it
void oracle_heat_update(float* heat, const float* new_heat, const float* active, const int* tet, float* vertex_heat,
                        int nt) {
    for (int t = 0; t < nt; ++t) {
        if (active[t] > 0.0f) {
            float h = new_heat[t];
            heat[t] = h;
            for (int k = 0; k < 4; ++k) vertex_heat[tet[4 * t + k]] = h / 4.0f;
        } else {
            heat[t] = 0.0f;
        }
    }
}

// checkTetrahedronHeat (integrator.py:874-895), or with rest volumes
// checkTetrahedronHeatVolumeProportional (integrator.py:897-918)
void oracle_check_heat(const float* heat, int* flip, const float* rest, const int* tet_tris, int* holes, float limit,
                       int nt) {
    for (int t = 0; t < nt; ++t) {
        bool hot = rest ? heat[t] > limit * rest[t] : heat[t] > limit;
        if (!hot || (!rest && flip[t] != 0)) continue;
        flip[t] = -1;
        for (int i = 0; i < 4; ++i)
            if (tet_tris[4 * t + i] > -1) holes[tet_tris[4 * t + i]] = 1;
    }
}

// heatLaparoscope (integrator.py:1153-1185): a serial read-add-write per triangle
void oracle_heat_laparoscope(const int* tri, const float* pos, const float* active, float* heat, const int* tri_tet,
                             const float* tips, const int* tri_env, float radius, float quantum, int nf) {
    for (int t = 0; t < nf; ++t) {
        int e = tri_env ? tri_env[t] : 0;
        V3<float> centre = (ld3<float>(tips, 4 * e + 1) + ld3<float>(tips, 4 * e + 2)) / 2.0f;
        V3<float> a = ld3<float>(pos, tri[3 * t]), b = ld3<float>(pos, tri[3 * t + 1]), c = ld3<float>(pos, tri[3 * t + 2]);
        V3<float> bary = closest_bary(a, b, c, centre);
        V3<float> closest = a * bary.x + b * bary.y + c * bary.z;
        if (length(closest - centre) < radius) {
            int k = tri_tet[t];
            if (k > -1 && active[k] > 0.0f) heat[k] = heat[k] + quantum;
        }
    }
}

// checkSegmentTriangleIntersection (integrator.py:1471-1518)
int oracle_segment_triangle(const float* pA_, const float* pB_, const float* pC_, const float* sA_, const float* sB_) {
    V3<float> pA = ld3<float>(pA_, 0), pB = ld3<float>(pB_, 0), pC = ld3<float>(pC_, 0);
    V3<float> sA = ld3<float>(sA_, 0), sB = ld3<float>(sB_, 0);
    V3<float> u = pB - pA, v = pC - pA, n = cross(u, v);
    if (n.x == 0.0f && n.y == 0.0f && n.z == 0.0f) return -1;
    V3<float> dir = sB - sA, w0 = sA - pA;
    float a = -dot(n, w0), b = dot(n, dir);
    if (std::fabs(b) < float(kFloatEpsilon)) return a == 0.0f ? 2 : 0;
    float r = a / b;
    if (r < 0.0f || r > 1.0f) return 0;
    V3<float> I = sA + r * dir;
    float uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
    V3<float> w = I - pA;
    float wu = dot(w, u), wv = dot(w, v);
    float D = uv * uv - uu * vv;
    float s = (uv * wv - vv * wu) / D;
    if (s < 0.0f || s > 1.0f) return 0;
    float tt = (uv * wu - uu * wv) / D;
    if (tt < 0.0f || (s + tt) > 1.0f) return 0;
    return 1;
}

// findIntersectingEdges (integrator.py:1406-1458): the triangle (rod tip, right clamp
// tip, left clamp tip) of the edge's env
void oracle_cut_edges(const float* pos, const float* tips, const int* edge, const float* active_edge, int* flip_edges,
                      int ne, const int* tet, int nt, const float* active_tet, int* flip_tets, const int* edge_tris,
                      int* holes, const int* edge_env) {
    for (int t = 0; t < ne; ++t) {
        int e = edge_env ? edge_env[t] : 0;
        int a = edge[2 * t], b = edge[2 * t + 1];
        const float* T0 = tips + 12ll * e;
        if (oracle_segment_triangle(T0, T0 + 6, T0 + 3, pos + 3ll * a, pos + 3ll * b) != 1) continue;
        if (flip_edges[t] == 0 && active_edge[t] == 1.0f) flip_edges[t] = -1;
        for (int k = 0; k < 2; ++k)
            if (edge_tris[2 * t + k] > -1) holes[edge_tris[2 * t + k]] = 1;
        for (int i = 0; i < nt; ++i)
            if (tet_holds(tet + 4 * i, a) && tet_holds(tet + 4 * i, b) && flip_tets[i] == 0 && active_tet[i] == 1.0f)
                flip_tets[i] = -1;
    }
}

// inDeCreaseActiveValues (integrator.py:1583-1605); counters beyond the table are left
// alone (the reference would read past it)
void oracle_update_active_values(int* flip, float* active, const float* table, int steps, int n) {
    for (int t = 0; t < n; ++t) {
        int f = flip[t];
        if (f == 0 || f > steps || f < -steps) continue;
        int k;
        if (f > 0) { k = f; flip[t] = f + 1; }
        else { k = steps + f; flip[t] = f - 1; }
        active[t] = table[k];
        if (std::abs(f) >= steps) flip[t] = 0;
    }
}

}  // extern "C"
