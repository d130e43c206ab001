// batched_kernel.cuh -- the env-resident batched step kernel, shared by the units that
// instantiate it under different compiler settings.
//
// One thread block owns one environment at a time and runs every substep and iteration
// of the step for it without leaving the SM: the env's predicted positions (with the
// inverse mass in .w) and its per-vertex correction accumulators live in shared memory,
// the read-only constraint tables stream from L2/HBM in coalesced structure-of-arrays
// records with 16-bit env-local vertex ids.  Blocks are persistent and take environments
// from a largest-first work list through an atomic counter, so meshes of uneven size
// share the GPU in one launch per size class.
//
// Semantics are SimIntegratorDO.stepModel's (FF_SRL/FF_SRL/integrator.py:1640-1741),
// Jacobi iteration unchanged: all constraint projections of an iteration read the same
// positions, their corrections are summed per vertex and divided by the number of
// contributing constraints (applyConstraints, integrator.py:946-960), then the grasp
// (dragConstraintsDO) and the instrument contact (collideLaparoscopeDO).
//
// Two arithmetic forms (template flag EX):
//  * reference (EX = true): every constraint is evaluated with the reference kernel's
//    expressions in its association order -- IEEE division and square root, F = Ds Dm^-1
//    for the Neo-Hookean constraint, no vertex reordering inside a tet -- and the unit is
//    compiled without multiply-add contraction, so each constraint's corrections are the
//    bits the serial restatement computes;
//  * fast (EX = false): one hardware reciprocal (rcp.approx) or reciprocal square root
//    per constraint, the Neo-Hookean constraint through M = Dm^-1 Dm^-T and the volume
//    cofactors, tet vertices reordered by even permutations so that folded edges sit at
//    fixed corners; compiled with contraction.
//
// Accumulation (storage policy S):
//  * AccFixed: each correction component, multiplied by the env's power-of-two scale, is
//    rounded once to a 32-bit fixed-point integer and summed with native shared-memory
//    integer atomics, which are associative: the sum does not depend on thread order, and
//    an environment gives the same bits alone or in any batch.  One unit is about a
//    quarter of a float ulp of the env's largest coordinate.  A term too large for the
//    32-bit per-vertex sum goes, exactly, to a 64-bit per-vertex side accumulator in
//    global memory that the next apply folds in, so no term is ever dropped; only a
//    non-finite term (or one beyond 2^62 units) flags the environment.  The number of
//    contributions per vertex is precomputed when the plan is built (a constraint only
//    skips at run time on degenerate geometry, which then decrements it), so no count
//    atomics are needed.
//  * AccKahan: per-vertex float32 (sum, compensation) pairs updated by a 64-bit
//    compare-and-swap loop: compensated (Kahan) summation of the corrections.
//  * AccAtomic: plain float32 atomics, as the reference's kernels accumulate.
//  * AccF64: the float64 build of the same kernel, summing in double.
// Constraint records are ordered by a greedy vertex colouring within each environment so
// that the 32 lanes of a warp update distinct vertices.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ffsrl_internal.h"

namespace ffsrl {
namespace bk {

#define BEPS 2.220446049250313e-16

template <class R> struct t3 { R x, y, z; };
template <class R> __device__ __forceinline__ t3<R> T3(R x, R y, R z) { t3<R> r; r.x = x; r.y = y; r.z = z; return r; }
template <class R> __device__ __forceinline__ t3<R> operator+(t3<R> a, t3<R> b) { return T3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> __device__ __forceinline__ t3<R> operator-(t3<R> a, t3<R> b) { return T3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> __device__ __forceinline__ t3<R> operator-(t3<R> a) { return T3<R>(-a.x, -a.y, -a.z); }
template <class R> __device__ __forceinline__ t3<R> operator*(t3<R> a, R s) { return T3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> __device__ __forceinline__ t3<R> operator*(R s, t3<R> a) { return T3<R>(s * a.x, s * a.y, s * a.z); }
template <class R> __device__ __forceinline__ t3<R> operator/(t3<R> a, R s) { return T3<R>(a.x / s, a.y / s, a.z / s); }
template <class R> __device__ __forceinline__ R dot(t3<R> a, t3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> __device__ __forceinline__ t3<R> cross(t3<R> a, t3<R> b) {
    return T3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> __device__ __forceinline__ R length(t3<R> a) { return sqrt(dot(a, a)); }
template <class R> __device__ __forceinline__ t3<R> normalize(t3<R> a) {
    R l = length(a);
    if (l > R(0)) return a / l;
    return T3<R>(0, 0, 0);
}
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
// Reciprocal and reciprocal square root of the fast form: one hardware approximation
// each in float32 (PTX rcp.approx / rsqrt.approx, about 1 ulp); exact in float64
__device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float rsqrt_(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double rsqrt_(double x) { return 1.0 / sqrt(x); }

// Brings the line holding p into this SM's L1 (PTX prefetch.global.L1); the tet loop
// requests the records its thread reads one loop trip later, so that read hits L1
// instead of waiting for L2
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// ---- accumulation policies ----------------------------------------------------------
struct AccFixed {
    typedef float R;
    typedef float4 P;
    typedef unsigned A;
    static constexpr bool kFixed = true;
    static constexpr bool kKahan = false;
};
struct AccKahan {
    typedef float R;
    typedef float4 P;
    typedef unsigned long long A;  // (sum bits | compensation bits << 32)
    static constexpr bool kFixed = false;
    static constexpr bool kKahan = true;
};
struct AccAtomic {
    typedef float R;
    typedef float4 P;
    typedef float A;
    static constexpr bool kFixed = false;
    static constexpr bool kKahan = false;
};
struct __align__(32) dpos { double x, y, z, w; };
struct AccF64 {
    typedef double R;
    typedef dpos P;
    typedef double A;
    static constexpr bool kFixed = false;
    static constexpr bool kKahan = false;
};

template <class R> struct PosOps;
template <> struct PosOps<float> {
    __device__ static t3<float> pos(const float4& p) { return T3<float>(p.x, p.y, p.z); }
    __device__ static float4 make(t3<float> v, float w) { return make_float4(v.x, v.y, v.z, w); }
};
template <> struct PosOps<double> {
    __device__ static t3<double> pos(const dpos& p) { return T3<double>(p.x, p.y, p.z); }
    __device__ static dpos make(t3<double> v, double w) { dpos r; r.x = v.x; r.y = v.y; r.z = v.z; r.w = w; return r; }
};

// Largest magnitude (in scaled units) a fixed-point term may take on the 64-bit side path
constexpr float kWideLimit = 4.611686e18f;  // 2^62

// Adds one scaled correction component `v` to accumulator word k.
template <class S> __device__ __forceinline__ void acc_add(typename S::A* acc, int k, typename S::R v);
template <> __device__ __forceinline__ void acc_add<AccFixed>(unsigned* acc, int k, float v) {
    atomicAdd(acc + k, (unsigned)__float2int_rn(v));
}
template <> __device__ __forceinline__ void acc_add<AccAtomic>(float* acc, int k, float v) { atomicAdd(acc + k, v); }
template <> __device__ __forceinline__ void acc_add<AccF64>(double* acc, int k, double v) { atomicAdd(acc + k, v); }
// Kahan step on the (sum, compensation) pair of word k: y = v - c; t = s + y;
// c' = (t - s) - y; s' = t, retried until no other thread changed the pair in between.
// The retries are capped: a pair still contended after 2^20 tries is set to NaN, which the
// step reports as a non-finite env instead of waiting on.
template <> __device__ __forceinline__ void acc_add<AccKahan>(unsigned long long* acc, int k, float v) {
    unsigned long long old = acc[k], assumed;
    int tries = 0;
    do {
        if (++tries > (1 << 20)) {
            atomicExch(acc + k, 0x7fc000007fc00000ull);
            return;
        }
        assumed = old;
        const float s = __uint_as_float((unsigned)(assumed & 0xffffffffull));
        const float c = __uint_as_float((unsigned)(assumed >> 32));
        const float y = v - c;
        const float t = s + y;
        const float cn = (t - s) - y;
        const unsigned long long nw = (unsigned long long)__float_as_uint(t) | ((unsigned long long)__float_as_uint(cn) << 32);
        old = atomicCAS(acc + k, assumed, nw);
    } while (old != assumed);
}
// The summed value of word k (in scaled units for AccFixed)
__device__ __forceinline__ float acc_value(const unsigned long long a) {
    return __uint_as_float((unsigned)(a & 0xffffffffull)) - __uint_as_float((unsigned)(a >> 32));
}

// Per-block context of the fixed-point side path
struct Wide {
    unsigned long long* w;  // [3V] per global vertex component, zero between uses
    long long v0;           // the env's first global vertex
    int* flag;              // shared: a term took the side path this phase
    float bound;            // largest scaled magnitude of one term on the 32-bit path
};

template <class R> __device__ __forceinline__ R abs_sum(t3<R> d) { return fabs(d.x) + fabs(d.y) + fabs(d.z); }

// Adds scaled correction vectors (already multiplied by the env's scale) to vertex i's
// accumulators.  `terms`: constraint contributions merged into this vector, each of which
// may use one term bound on the 32-bit path.  AccFixed: a vector beyond that bound goes to
// the 64-bit side accumulator (exact); a non-finite one raises `bad`.
template <class S> __device__ __forceinline__ void add3s(typename S::A* acc, int i, t3<typename S::R> d, bool& bad,
                                                         const Wide& wd, typename S::R terms) {
    typedef typename S::R R;
    if constexpr (S::kFixed) {
        if (abs_sum(d) < wd.bound * terms) {
            acc_add<S>(acc, 3 * i, d.x); acc_add<S>(acc, 3 * i + 1, d.y); acc_add<S>(acc, 3 * i + 2, d.z);
            return;
        }
        const R c[3] = {d.x, d.y, d.z};
        for (int k = 0; k < 3; ++k) {
            if (!(fabsf(c[k]) < kWideLimit)) { bad = true; continue; }
            atomicAdd(wd.w + 3 * (wd.v0 + i) + k, (unsigned long long)__float2ll_rn(c[k]));
        }
        *wd.flag = 1;
    } else {
        (void)wd; (void)terms;
        if (!isfinite(abs_sum(d))) bad = true;
        acc_add<S>(acc, 3 * i, d.x); acc_add<S>(acc, 3 * i + 1, d.y); acc_add<S>(acc, 3 * i + 2, d.z);
    }
}

// Reads and clears vertex i's three sums (value in model units); AccFixed folds in the
// side accumulator when the phase used it, and `extra` (pending connector sums, scaled)
template <class S> __device__ __forceinline__ t3<typename S::R> take3(typename S::A* acc, int i, bool wide_on,
                                                                      const Wide& wd, float inv, const long long* extra) {
    typedef typename S::R R;
    t3<R> r;
    if constexpr (S::kFixed) {
        if (!wide_on && !extra) {
            // the common case: the 32-bit sum alone (int32 -> float, the same rounding as the
            // 64-bit conversion below, which runs on the slow float64 unit)
            r = T3<R>(__int2float_rn((int)acc[3 * i]) * inv, __int2float_rn((int)acc[3 * i + 1]) * inv,
                      __int2float_rn((int)acc[3 * i + 2]) * inv);
        } else {
            long long s[3];
            for (int k = 0; k < 3; ++k) s[k] = (long long)(int)acc[3 * i + k];
            if (wide_on) {
                unsigned long long* w = wd.w + 3 * (wd.v0 + i);
                for (int k = 0; k < 3; ++k) { s[k] += (long long)w[k]; w[k] = 0ull; }
            }
            if (extra)
                for (int k = 0; k < 3; ++k) s[k] += extra[k];
            r = T3<R>(__ll2float_rn(s[0]) * inv, __ll2float_rn(s[1]) * inv, __ll2float_rn(s[2]) * inv);
        }
    } else if constexpr (S::kKahan) {
        r = T3<R>(acc_value(acc[3 * i]), acc_value(acc[3 * i + 1]), acc_value(acc[3 * i + 2]));
    } else {
        r = T3<R>(acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]);
    }
    acc[3 * i] = typename S::A(0); acc[3 * i + 1] = typename S::A(0); acc[3 * i + 2] = typename S::A(0);
    return r;
}

// v0/nv: the env's vertices in the model arrays; t0/e0/f0: its constraint tables, which
// envs with identical tables share; mt0/me0: its tets/edges in the model arrays (for the
// XPBD multipliers, which are per env); sc/inv: the env's fixed-point scale (a power of
// two) and its inverse
struct EnvRec { int v0, nv, t0, nt, e0, ne, f0, nf, mt0, me0, c0, nc; float sc, inv; };

template <class R> struct Dev {
    const EnvRec* env;
    const uint2* tet_idx;      // 4 x u16 local ids
    const float2* tet_va;      // (|V0|, active)
    const float4* nh0;         // fast Neo-Hookean: M = Dm^-1 Dm^-T entries (00, 01, 02, 11)
    const float4* nh1;         // (M12, M22, det Dm^-1, 1/|V0|)
    const float4* nhd;         // reference Neo-Hookean: Dm^-1 row-major in 3 float4 per tet (9 used)
    const float* tet_vs;       // signed rest volume (XPBD)
    const unsigned* edge_idx;  // 2 x u16 local ids
    const float2* edge_la;     // (L0, active)
    const uint2* tri_idx;      // (a | b<<16, c | hole<<16)
    R* vertex; R* velocity; R* predicted;
    const float* inv_mass; const float* drag;
    const float* lap_base; const float* lap_tip; const float* lap_radius;
    int* in_collision;
    float* tet_lambda; float* edge_lambda;
    int* env_status;
    const int* cnt0;           // per-vertex static contribution count (global vertex index)
    const float4* tet_ed;      // distance constraints solved by the tet: (L0 of A-B, active, +-L0, active);
                               // the second is C-D for +L0 and A-C for -L0; active 0 = none
    const float2* tet_ed2;     // compact records: (L0 of A-B, +-L0 of C-D / A-C), 0 = none, active 1
    int fold;                  // distance constraints folded into the tet records
    int compact;               // compact fast-form records: no tet_va, nh1.w = +-|V0| (sign: active),
                               // folded edges in tet_ed2
    const uint2* conn_idx;     // connectors: (point | triangle a << 16, b | c << 16), env-local ids
    const float4* conn_bar;    // (barycentric 0, 1, 2, rest distance)
    const unsigned char* conn_vert;  // per vertex (global id): 1 when a connector holds it
    long long* pend;           // [3V] connector corrections waiting for the next apply (fixed point)
    int* pcnt;                 // [V] their counts
    unsigned long long* wide;  // [3V] fixed-point side accumulator
    float bound;               // scaled magnitude one term may take on the 32-bit path
    float conn_w, conn_ks, conn_mul;  // mass weight ratio, kS, rest length multiplier
    const int* tet_orig;       // env-local model tet id of each (colour-ordered) record, for XPBD lambdas
    const int* edge_orig;      // env-local model edge id of each record
    unsigned flags;
    int substeps, iterations;
    float dt, gx, gy, gz, damping, ground;
    float ks_distance, ks_volume, ks_contact, ks_drag;
    float vol_c, dev_c, a_dist, a_vol;
};

template <class R> __device__ __forceinline__ t3<R> ldgen3(const R* p, long long i) { return T3<R>(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
template <class R> __device__ __forceinline__ void stg3(R* p, long long i, t3<R> v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }
__device__ __forceinline__ t3<float> ldf3(const float* __restrict__ p, long long i) {
    return T3<float>(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2));
}
template <class R> __device__ __forceinline__ t3<R> prom(t3<float> a) { return T3<R>(R(a.x), R(a.y), R(a.z)); }

// closestPointOnEdge (integrator.py:1520-1534)
template <class R> __device__ __forceinline__ t3<R> closest_on_edge(t3<R> p, t3<R> a, t3<R> b) {
    t3<R> d = b - a;
    R t;
    if (length(d) < R(BEPS)) {
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
template <class R> __device__ __forceinline__ t3<R> closest_bary(t3<R> a, t3<R> b, t3<R> c, t3<R> p) {
    t3<R> ab = b - a, ac = c - a, ap = p - a;
    R d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= R(0) && d2 <= R(0)) return T3<R>(1, 0, 0);
    t3<R> bp = p - b;
    R d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= R(0) && d4 <= d3) return T3<R>(0, 1, 0);
    R vc = d1 * d4 - d3 * d2;
    R v = d1 / (d1 - d3);
    if (vc <= R(0) && d1 >= R(0) && d3 <= R(0)) return T3<R>(R(1) - v, v, 0);
    t3<R> cp = p - c;
    R d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= R(0) && d5 <= d6) return T3<R>(0, 0, 1);
    R vb = d5 * d2 - d1 * d6;
    R w = d2 / (d2 - d6);
    if (vb <= R(0) && d2 >= R(0) && d6 <= R(0)) return T3<R>(R(1) - w, 0, w);
    R va = d3 * d6 - d5 * d4;
    w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    if (va <= R(0) && (d4 - d3) >= R(0) && (d5 - d6) >= R(0)) return T3<R>(0, w, R(1) - w);
    R denom = R(1) / (va + vb + vc);
    v = vb * denom;
    w = vc * denom;
    return T3<R>(R(1) - v - w, v, w);
}

// checkSdfCapsuleCollision (integrator.py:1302-1355)
template <class R> __device__ __forceinline__ bool capsule_response(t3<R> tip, t3<R> base, R radius, t3<R> n,
                                                                    t3<R> centre, t3<R> pA, t3<R> pB, t3<R> pC, R ks,
                                                                    t3<R>& rA, t3<R>& rB, t3<R>& rC) {
    t3<R> cn = normalize(tip - base);
    t3<R> off = cn * radius;
    t3<R> posA = base + off;
    t3<R> posB = tip - off;
    R denom = dot(n, cn);
    if (fabs(denom) < R(BEPS)) return false;
    R t = dot(n, centre - base) / denom;
    t3<R> lp = base + cn * t;
    t3<R> ref = closest_bary(pA, pB, pC, lp);
    t3<R> sc = closest_on_edge(ref, posA, posB);
    t3<R> bary = closest_bary(pA, pB, pC, sc);
    t3<R> contact = pA * bary.x + pB * bary.y + pC * bary.z;
    t3<R> sv = sc - contact;
    R dist = length(sv);
    R pen = radius / length(sv) - R(1);
    t3<R> pv = T3<R>(pen * sv.x, pen * sv.y, pen * sv.z);
    R plen = length(pv);
    t3<R> pn = normalize(pv);
    R sq = bary.x * bary.x + bary.y * bary.y + bary.z * bary.z;
    if (sq < R(BEPS)) return false;
    t3<R> resp = pn * (plen / sq) * ks;
    if (dist > radius) return false;
    rA = resp * bary.x; rB = resp * bary.y; rC = resp * bary.z;
    return true;
}

// One distance constraint (distanceConstraints, integrator.py:65-109) between two of a
// tet's vertices u and v, added to the tet's corrections (u gets -d m_u, v gets +d m_v),
// multiplied by the scale `sc`.  Returns 1 when it contributed.  A degenerate length
// decrements the two static counts and records the iteration in *dyn_it.  EX: the
// reference's expression, -C (dir/len) kS active / w per component; the result is the
// same whichever end the model lists first (each step is sign-symmetric).
template <bool EX, class R> __device__ __forceinline__ int fold_edge(t3<R> pu, t3<R> pv, R mu, R mv, R L0, R active,
                                                                     t3<R>& du, t3<R>& dv, int iu, int iv, int* cnt,
                                                                     int it, R ks, int* dyn_it, R sc) {
    const R w = mu + mv;
    if (w < R(BEPS)) return 0;  // never counted
    const t3<R> dir = pv - pu;
    const R dd = dot(dir, dir);
    if constexpr (EX) {
        const R len = sqrt(dd);
        if (len < R(BEPS)) {
            atomicSub(cnt + iu, 1); atomicSub(cnt + iv, 1);
            *dyn_it = it;
            return 0;
        }
        const R C = len - L0;
        const t3<R> d = -C * (dir / len) * ks * active / w;
        du = du - (d * mu) * sc;
        dv = dv + (d * mv) * sc;
    } else {
        if (dd < R(BEPS * BEPS)) {
            atomicSub(cnt + iu, 1); atomicSub(cnt + iv, 1);
            *dyn_it = it;
            return 0;
        }
        const R rl = rsqrt_(dd);
        const R C = dd * rl - L0;
        const t3<R> d = dir * (-C * rl * ks * active * rcp(w) * sc);
        du = du - d * mu;
        dv = dv + d * mv;
    }
    return 1;
}

template <class R> struct ToolShared {
    t3<R> base[3], tip[3];
    R radius[3];
    t3<R> blo[3], bhi[3];  // conservative contact boxes per capsule
    t3<R> ulo, uhi;        // their union
    t3<R> drag_tip;
};

// near-contact triangles an iteration's scan hands to the whole block (entries: triangle
// << 3 | capsule mask); more than this are solved by the thread that found them
constexpr int kNearCap = 512;

// Dynamic shared memory of a block: its env state (positions and inverse masses, the
// accumulators and counts in MODE 0) for up to max_nv vertices, then the grasp bits; a
// class may add its envs' surface triangles behind that (8-byte aligned)
template <class S> __host__ __device__ size_t smem_bytes(int mode, int max_nv) {
    size_t P = sizeof(typename S::P), A = sizeof(typename S::A);
    size_t bits = 4 * (size_t)((max_nv + 31) / 32 + 1);
    if (mode == 0) {
        // counts after the accumulators; keep the grasp bits 4-byte aligned
        return (P + 3 * A + 4) * (size_t)max_nv + bits;
    }
    if (mode == 1) return P * (size_t)max_nv + bits;
    return bits;
}
template <class S> size_t scratch_bytes(int mode, int max_nv) {
    size_t P = sizeof(typename S::P), A = sizeof(typename S::A);
    if (mode == 0) return 0;
    if (mode == 1) return (3 * A + 4) * (size_t)max_nv;
    return (P + 3 * A + 4) * (size_t)max_nv;
}

// The constraint set of config 1 and the mixed pools, fixed at compile time in their own
// instantiations
constexpr unsigned kLiverFlags = FFSRL_VOLUME | FFSRL_DISTANCE | FFSRL_NEOHOOKEAN | FFSRL_DRAG | FFSRL_COLLIDE;

// One tet's records
struct TetRec {
    uint2 ix;
    float2 va;
    float4 n0, n1, n2, ed;
};

template <bool EX, bool NH, bool FOLD, class R>
__device__ __forceinline__ TetRec load_tet(const Dev<R>& D, long long g) {
    TetRec r;
    r.ix = __ldg(D.tet_idx + g);
    r.n0 = r.n1 = r.n2 = r.ed = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!EX && NH && FOLD && D.compact) {
        // 48 bytes a tet instead of 64: |V0| and the volume constraint's activity ride in
        // the sign of nh1.w, 1/|V0| is formed here, folded edges are always active
        r.n0 = __ldg(D.nh0 + g);
        r.n1 = __ldg(D.nh1 + g);
        const float2 e = __ldg(D.tet_ed2 + g);
        const float v0 = fabsf(r.n1.w);
        r.va = make_float2(v0, signbit(r.n1.w) ? 0.0f : 1.0f);
        r.n1.w = rcp(v0);
        r.ed = make_float4(e.x, e.x != 0.0f ? 1.0f : 0.0f, e.y, e.y != 0.0f ? 1.0f : 0.0f);
        return r;
    }
    r.va = __ldg(D.tet_va + g);
    if (NH) {
        if (EX) { r.n0 = __ldg(D.nhd + 3 * g); r.n1 = __ldg(D.nhd + 3 * g + 1); r.n2 = __ldg(D.nhd + 3 * g + 2); }
        else { r.n0 = __ldg(D.nh0 + g); r.n1 = __ldg(D.nh1 + g); }
    }
    if (FOLD) r.ed = __ldg(D.tet_ed + g);
    return r;
}
template <bool EX, class R>
__device__ __forceinline__ TetRec load_tet_sel(const Dev<R>& D, long long g, bool nh, bool fold) {
    return nh ? (fold ? load_tet<EX, true, true>(D, g) : load_tet<EX, true, false>(D, g))
              : (fold ? load_tet<EX, false, true>(D, g) : load_tet<EX, false, false>(D, g));
}

// MODE 0: positions and accumulators in shared memory.  MODE 1: positions in shared
// memory, accumulators in the block's global scratch.  MODE 2: both in global scratch.
// PIPE: the tet loop holds the thread's next tet record in registers, loaded while the
// current one is solved (for block sizes that leave the registers for it).
// FL: the constraint selection fixed at compile time (0: read from the parameters).
template <class S, int BLOCK, int MODE, bool PIPE = false, unsigned FL = 0, bool EX = false>
__global__ void __launch_bounds__(BLOCK, (BLOCK <= 256 ? 768 / BLOCK : 1))
    k_batched(const Dev<typename S::R> D, const int* __restrict__ work, int nwork, int* counter, int nsteps,
              unsigned char* scratch, long long scratch_stride, int max_nv, int prefetch, int tri_cap) {
    typedef typename S::R R;
    typedef typename S::P P;
    typedef typename S::A A;
    typedef PosOps<R> PO;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_work;
    __shared__ int s_incol;
    __shared__ int s_bad;
    __shared__ int s_any_contact;
    __shared__ int s_any_drag;
    __shared__ int s_dyn_it;  // iteration in which a constraint skipped on degenerate geometry
    __shared__ int s_near_n;
    __shared__ int s_wide_c[2];  // a fixed-point term took the 64-bit side path in the constraint phase
                                 // of an iteration of this parity
    __shared__ int s_wide_k;  // ... in the contact phase
    __shared__ unsigned s_near[kNearCap];
    __shared__ ToolShared<R> tool;

    unsigned char* gbase = scratch + (long long)blockIdx.x * scratch_stride;
    const int tid = threadIdx.x;
    const R dt = R(D.dt);
    const unsigned fl = FL ? FL : D.flags;
    const bool has_conn = (fl & FFSRL_CONNECTORS) && D.conn_idx != nullptr;
    // Neo-Hookean constants, hoisted with the reference's association order (the same
    // operations on the same values give the same bits): C offset invDev/invVol, and
    // compliance/dT/dT (the per-tet /V0 stays per tet)
    const R nh_off = (R(1) / R(D.dev_c)) / (R(1) / R(D.vol_c));
    const R nh_uH = R(D.vol_c) / dt / dt;
    const R nh_uD = R(D.dev_c) / dt / dt;

    for (;;) {
        // the per-env flags are cleared before the barrier: after it, any warp may set them
        // (the grasp bits below set s_any_drag from every warp)
        if (tid == 0) {
            s_work = atomicAdd(counter, 1);
            s_incol = 0; s_bad = 0; s_any_drag = 0; s_dyn_it = -1; s_wide_c[0] = 0; s_wide_c[1] = 0; s_wide_k = 0;
        }
        __syncthreads();
        const int w = s_work;
        if (w >= nwork) return;
        const int env = work[w];
        const EnvRec E = D.env[env];
        const int nv = E.nv, nt = E.nt, ne = E.ne, nf = E.nf;
        const R sc = S::kFixed ? R(E.sc) : R(1);  // power of two: scaling a product by it is exact
        const float inv_sc = E.inv;
        const Wide wk{D.wide, (long long)E.v0, &s_wide_k, D.bound};  // contact phase

        P* xp;
        A* acc;
        int* cnt;
        unsigned* dbits;
        if (MODE == 0) {
            xp = reinterpret_cast<P*>(smem);
            acc = reinterpret_cast<A*>(smem + sizeof(P) * (size_t)max_nv);
            cnt = reinterpret_cast<int*>(smem + (sizeof(P) + 3 * sizeof(A)) * (size_t)max_nv);
            dbits = reinterpret_cast<unsigned*>(smem + (sizeof(P) + 3 * sizeof(A) + sizeof(int)) * (size_t)max_nv);
        } else if (MODE == 1) {
            xp = reinterpret_cast<P*>(smem);
            dbits = reinterpret_cast<unsigned*>(smem + sizeof(P) * (size_t)max_nv);
            acc = reinterpret_cast<A*>(gbase);
            cnt = reinterpret_cast<int*>(gbase + 3 * sizeof(A) * (size_t)max_nv);
        } else {
            dbits = reinterpret_cast<unsigned*>(smem);
            xp = reinterpret_cast<P*>(gbase);
            acc = reinterpret_cast<A*>(gbase + sizeof(P) * (size_t)max_nv);
            cnt = reinterpret_cast<int*>(gbase + (sizeof(P) + 3 * sizeof(A)) * (size_t)max_nv);
        }

        bool bad = false;
        if (tid == 0) {
            for (int i = 0; i < 3; ++i) {
                long long k = 4ll * env + i;
                t3<R> b = prom<R>(ldf3(D.lap_base, k)), t = prom<R>(ldf3(D.lap_tip, k));
                R r = R(D.lap_radius[k]);
                tool.base[i] = b; tool.tip[i] = t; tool.radius[i] = r;
                t3<R> cn = normalize(t - b);
                t3<R> off = cn * r;
                t3<R> pa = b + off, pb = t - off;
                R mag = rmax(rmax(rmax(fabs(pa.x), fabs(pa.y)), rmax(fabs(pa.z), fabs(pb.x))),
                             rmax(fabs(pb.y), fabs(pb.z)));
                R m = r + R(1e-4) * (R(1) + mag);
                tool.blo[i] = T3<R>(rmin(pa.x, pb.x) - m, rmin(pa.y, pb.y) - m, rmin(pa.z, pb.z) - m);
                tool.bhi[i] = T3<R>(rmax(pa.x, pb.x) + m, rmax(pa.y, pb.y) + m, rmax(pa.z, pb.z) + m);
                if (i == 2) tool.drag_tip = t;
            }
            tool.ulo = T3<R>(rmin(tool.blo[0].x, rmin(tool.blo[1].x, tool.blo[2].x)),
                             rmin(tool.blo[0].y, rmin(tool.blo[1].y, tool.blo[2].y)),
                             rmin(tool.blo[0].z, rmin(tool.blo[1].z, tool.blo[2].z)));
            tool.uhi = T3<R>(rmax(tool.bhi[0].x, rmax(tool.bhi[1].x, tool.bhi[2].x)),
                             rmax(tool.bhi[0].y, rmax(tool.bhi[1].y, tool.bhi[2].y)),
                             rmax(tool.bhi[0].z, rmax(tool.bhi[1].z, tool.bhi[2].z)));
        }
        for (int i = tid; i < nv; i += BLOCK) {
            acc[3 * i] = A(0); acc[3 * i + 1] = A(0); acc[3 * i + 2] = A(0);
            cnt[i] = __ldg(D.cnt0 + E.v0 + i);
        }
        // grasp mask of this env, one bit per vertex
        if (fl & FFSRL_DRAG) {
            const int lane = tid & 31;
            for (int b0 = tid & ~31; b0 < nv; b0 += BLOCK) {
                int i = b0 + lane;
                bool on = i < nv && __ldg(D.drag + E.v0 + i) != 0.0f;
                unsigned word = __ballot_sync(0xffffffffu, on);
                if (lane == 0) {
                    dbits[b0 >> 5] = word;
                    if (word) s_any_drag = 1;
                }
            }
        }
        // the env's surface triangles, when the class keeps them in shared memory
        uint2* tri_s = nullptr;
        if (tri_cap) {
            tri_s = reinterpret_cast<uint2*>(smem + ((smem_bytes<S>(MODE, max_nv) + 7) & ~(size_t)7));
            for (int f = tid; f < nf; f += BLOCK) tri_s[f] = __ldg(D.tri_idx + (long long)E.f0 + f);
        }
        // inverse masses ride in .w for the whole step
        for (int i = tid; i < nv; i += BLOCK) {
            t3<R> x = ldgen3(D.vertex, E.v0 + i);
            xp[i] = PO::make(x, R(__ldg(D.inv_mass + E.v0 + i)));
        }
        __syncthreads();

        for (int step = 0; step < nsteps; ++step) {
            for (int sub = 0; sub < D.substeps; ++sub) {
                // gravity (integrator.py:40-63)
                for (int i = tid; i < nv; i += BLOCK) {
                    t3<R> x = ldgen3(D.vertex, E.v0 + i), v = ldgen3(D.velocity, E.v0 + i);
                    R inv = xp[i].w;
                    R damp = R(1) - R(D.damping);
                    v = v + T3<R>(R(D.gx), R(D.gy), R(D.gz)) * inv * dt * damp;
                    if (inv < R(BEPS)) v = T3<R>(0, 0, 0);
                    xp[i] = PO::make(x + v * dt, inv);
                }
                if (fl & FFSRL_VOLUME_XPBD)
                    for (int t = tid; t < nt; t += BLOCK) D.tet_lambda[E.mt0 + t] = 0.0f;
                if (fl & FFSRL_DISTANCE_XPBD)
                    for (int e = tid; e < ne; e += BLOCK) D.edge_lambda[E.me0 + e] = 0.0f;
                __syncthreads();

                for (int it = 0; it < D.iterations; ++it) {
                    // The constraint phase's side-path flag alternates by iteration parity: the
                    // apply of iteration j clears the flag iteration j + 1 will set, while no
                    // thread can still be setting or reading it (those phases lie behind or
                    // ahead of a barrier), so a set flag is never lost.  A stale set flag only
                    // costs the apply a read of zeros.
                    const Wide wd{D.wide, (long long)E.v0, &s_wide_c[it & 1], D.bound};
                    // ---- tet constraints: volume, XPBD volume, Neo-Hookean ----
                    if (fl & (FFSRL_VOLUME | FFSRL_VOLUME_XPBD | FFSRL_NEOHOOKEAN)) {
                        const bool nhf = (fl & FFSRL_NEOHOOKEAN) != 0;
                        const bool fold = D.fold != 0;
                        TetRec nx;
                        if (PIPE && tid < nt) {
                            const long long g0 = E.t0 + tid;
                            nx = load_tet_sel<EX>(D, g0, nhf, fold);
                        }
                        for (int t = tid; t < nt; t += BLOCK) {
                            const long long gt = E.t0 + t;
                            TetRec rc;
                            if (PIPE) {
                                rc = nx;
                                if (t + BLOCK < nt) {  // the next record, in flight while this tet is solved
                                    const long long gn = gt + BLOCK;
                                    nx = load_tet_sel<EX>(D, gn, nhf, fold);
                                }
                            } else {
                                if (prefetch && t + BLOCK < nt) {  // this thread's next record, into L1
                                    const long long gn = gt + BLOCK;
                                    prefetch_l1(D.tet_idx + gn);
                                    if (EX || !D.compact) prefetch_l1(D.tet_va + gn);
                                    if (nhf) {
                                        if (EX) { prefetch_l1(D.nhd + 3 * gn); prefetch_l1(D.nhd + 3 * gn + 2); }
                                        else { prefetch_l1(D.nh0 + gn); prefetch_l1(D.nh1 + gn); }
                                    }
                                    if (fold) {
                                        if (!EX && D.compact) prefetch_l1(D.tet_ed2 + gn);
                                        else prefetch_l1(D.tet_ed + gn);
                                    }
                                }
                                // every record of the tet is requested up front, so its loads are in
                                // flight together
                                rc = load_tet_sel<EX>(D, gt, nhf, fold);
                            }
                            const uint2 ix = rc.ix;
                            const float2 va = rc.va;
                            const float4 ed = rc.ed;
                            const int ia = ix.x & 0xffff, ib = ix.x >> 16, ic = ix.y & 0xffff, id = ix.y >> 16;
                            const P PA = xp[ia], PB = xp[ib], PC = xp[ic], PD = xp[id];
                            const t3<R> pa = PO::pos(PA), pb = PO::pos(PB), pc = PO::pos(PC), pd = PO::pos(PD);
                            const R mA = PA.w, mB = PB.w, mC = PC.w, mD = PD.w;
                            const t3<R> p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
                            t3<R> dA = T3<R>(0, 0, 0), dB = dA, dC = dA, dD = dA;
                            int k = 0;     // constraints that contributed
                            int skip = 0;  // statically counted constraints that skipped on degenerate geometry
                            const bool anym = mA != R(0) || mB != R(0) || mC != R(0) || mD != R(0);
                            // cofactor columns of Ds = [p1 p2 p3]: the volume gradient, and (times det Dm^-1) the
                            // fast Neo-Hookean hydrostatic gradient cof(F) Dm^-T = det(Dm^-1) cof(Ds)
                            const t3<R> q1 = cross(p2, p3), q2 = cross(p3, p1), q3 = cross(p1, p2);
                            const t3<R> q0 = -q1 - q2 - q3;
                            const R wq = mA * dot(q0, q0) + mB * dot(q1, q1) + mC * dot(q2, q2) + mD * dot(q3, q3);
                            const R s6 = dot(q3, p3);  // det Ds = 6 x signed volume
                            if (fl & (FFSRL_VOLUME | FFSRL_VOLUME_XPBD)) {
                                // volumeConstraints (integrator.py:444-504) / XPBD (:507-576)
                                const R active = R(va.y);
                                if (active == R(1)) {
                                    if (fabs(wq) < R(BEPS)) {
                                        if (anym) skip += ((fl & FFSRL_VOLUME) ? 1 : 0) + ((fl & FFSRL_VOLUME_XPBD) ? 1 : 0);
                                    } else {
                                        if (fl & FFSRL_VOLUME) {
                                            if constexpr (EX) {
                                                const R vol = fabs(s6) / R(6);
                                                const R C = R(va.x) - vol;
                                                const R dl = -R(D.ks_volume) * active * C / wq;
                                                dA = (q0 * dl * mA) * sc; dB = (q1 * dl * mB) * sc;
                                                dC = (q2 * dl * mC) * sc; dD = (q3 * dl * mD) * sc;
                                            } else {
                                                R C = R(va.x) - fabs(s6) * R(1.0 / 6.0);
                                                const R dl = -R(D.ks_volume) * active * C * rcp(wq) * sc;
                                                dA = q0 * dl * mA; dB = q1 * dl * mB; dC = q2 * dl * mC; dD = q3 * dl * mD;
                                            }
                                            ++k;
                                        }
                                        if (fl & FFSRL_VOLUME_XPBD) {
                                            R alpha = R(D.a_vol);
                                            const int ot = E.mt0 + __ldg(D.tet_orig + gt);
                                            R lam = R(D.tet_lambda[ot]);
                                            R C = s6 / R(6) - R(__ldg(D.tet_vs + gt));
                                            R dl = -(C + alpha * lam) / (wq + alpha);
                                            D.tet_lambda[ot] = float(lam + dl);
                                            dA = dA + (q0 * dl * mA) * sc; dB = dB + (q1 * dl * mB) * sc;
                                            dC = dC + (q2 * dl * mC) * sc; dD = dD + (q3 * dl * mD) * sc;
                                            ++k;
                                        }
                                    }
                                }
                            }
                            if (fl & FFSRL_NEOHOOKEAN) {
                                if constexpr (EX) {
                                    // neoHookeanConstraints (integrator.py:578-698): F = Ds Dm^-1 by
                                    // columns, hydrostatic gradient from the cofactor columns of F
                                    // times Dm^-T, deviatoric from F Dm^-T / |F|, each with the
                                    // reference's lambda-free compliant update
                                    const R D00 = R(rc.n0.x), D01 = R(rc.n0.y), D02 = R(rc.n0.z);
                                    const R D10 = R(rc.n0.w), D11 = R(rc.n1.x), D12 = R(rc.n1.y);
                                    const R D20 = R(rc.n1.z), D21 = R(rc.n1.w), D22 = R(rc.n2.x);
                                    const R rv = R(va.x);
                                    const t3<R> f0 = p1 * D00 + p2 * D10 + p3 * D20;
                                    const t3<R> f1 = p1 * D01 + p2 * D11 + p3 * D21;
                                    const t3<R> f2 = p1 * D02 + p2 * D12 + p3 * D22;
                                    const t3<R> c0 = cross(f1, f2), c1 = cross(f2, f0), c2 = cross(f0, f1);
                                    t3<R> g1 = c0 * D00 + c1 * D01 + c2 * D02;
                                    t3<R> g2 = c0 * D10 + c1 * D11 + c2 * D12;
                                    t3<R> g3 = c0 * D20 + c1 * D21 + c2 * D22;
                                    t3<R> g0 = -g1 - g2 - g3;
                                    const R detF = dot(f0, c0);
                                    R C = detF - R(1) - nh_off;
                                    R wn = R(0), l;
                                    l = length(g0); wn += l * l * mA;
                                    l = length(g1); wn += l * l * mB;
                                    l = length(g2); wn += l * l * mC;
                                    l = length(g3); wn += l * l * mD;
                                    if (wn < R(BEPS)) {
                                        if (anym) ++skip;
                                    } else {
                                        R dl = -C / (wn + nh_uH / rv);
                                        t3<R> nA = g0 * dl * mA, nB = g1 * dl * mB, nC = g2 * dl * mC, nD = g3 * dl * mD;
                                        const R l0 = length(f0), l1 = length(f1), l2 = length(f2);
                                        const R rs = sqrt(l0 * l0 + l1 * l1 + l2 * l2);
                                        const R rsi = R(1) / rs;
                                        C = rs;
                                        g1 = (f0 * D00 + f1 * D01 + f2 * D02) * rsi;
                                        g2 = (f0 * D10 + f1 * D11 + f2 * D12) * rsi;
                                        g3 = (f0 * D20 + f1 * D21 + f2 * D22) * rsi;
                                        g0 = -g1 - g2 - g3;
                                        wn = R(0);
                                        l = length(g0); wn += l * l * mA;
                                        l = length(g1); wn += l * l * mB;
                                        l = length(g2); wn += l * l * mC;
                                        l = length(g3); wn += l * l * mD;
                                        if (wn < R(BEPS)) {
                                            if (anym) ++skip;
                                        } else {
                                            dl = -C / (wn + nh_uD / rv);
                                            nA = nA + g0 * dl * mA; nB = nB + g1 * dl * mB;
                                            nC = nC + g2 * dl * mC; nD = nD + g3 * dl * mD;
                                            dA = dA + nA * sc; dB = dB + nB * sc; dC = dC + nC * sc; dD = dD + nD * sc;
                                            ++k;
                                        }
                                    }
                                } else {
                                    // neoHookeanConstraints (integrator.py:578-698) with F = Ds Dm^-1 written through
                                    // M = Dm^-1 Dm^-T: |F|^2 = sum_ij (Ds^T Ds)_ij M_ij, F Dm^-T = Ds M, det F = det Ds det Dm^-1
                                    const R m00 = R(rc.n0.x), m01 = R(rc.n0.y), m02 = R(rc.n0.z), m11 = R(rc.n0.w);
                                    const R m12 = R(rc.n1.x), m22 = R(rc.n1.y), detD = R(rc.n1.z), inv_rv = R(rc.n1.w);
                                    const R C = s6 * detD - R(1) - nh_off;
                                    const R wH = wq * detD * detD;
                                    if (wH < R(BEPS)) {
                                        if (anym) ++skip;
                                    } else {
                                        const R dlH = -C * rcp(wH + nh_uH * inv_rv);
                                        const R rs2 = dot(p1, p1) * m00 + dot(p2, p2) * m11 + dot(p3, p3) * m22 +
                                                      R(2) * (dot(p1, p2) * m01 + dot(p1, p3) * m02 + dot(p2, p3) * m12);
                                        const R rsi = rsqrt_(rs2);
                                        const R rs = rs2 * rsi;
                                        const t3<R> e1 = p1 * m00 + p2 * m01 + p3 * m02;
                                        const t3<R> e2 = p1 * m01 + p2 * m11 + p3 * m12;
                                        const t3<R> e3 = p1 * m02 + p2 * m12 + p3 * m22;
                                        const t3<R> e0 = -e1 - e2 - e3;
                                        const R wD = (mA * dot(e0, e0) + mB * dot(e1, e1) + mC * dot(e2, e2) + mD * dot(e3, e3)) * (rsi * rsi);
                                        if (wD < R(BEPS)) {
                                            if (anym) ++skip;
                                        } else {
                                            const R ce = -rs * rcp(wD + nh_uD * inv_rv) * rsi * sc;
                                            const R ch = dlH * detD * sc;
                                            dA = dA + (q0 * (ch * mA) + e0 * (ce * mA)); dB = dB + (q1 * (ch * mB) + e1 * (ce * mB));
                                            dC = dC + (q2 * (ch * mC) + e2 * (ce * mC)); dD = dD + (q3 * (ch * mD) + e3 * (ce * mD));
                                            ++k;
                                        }
                                    }
                                }
                            }
                            const int ktet = k;  // tet constraints merged into each vertex's term
                            if (fold) {
                                // distanceConstraints (integrator.py:65-109) of the edges this tet solves:
                                // A-B in the first slot, C-D (+L0) or A-C (-L0) in the second
                                if (ed.y != 0.0f) k += fold_edge<EX, R>(pa, pb, mA, mB, R(ed.x), R(ed.y), dA, dB, ia, ib, cnt, it, R(D.ks_distance), &s_dyn_it, sc);
                                if (ed.w != 0.0f) {
                                    if (ed.z > 0.0f) k += fold_edge<EX, R>(pc, pd, mC, mD, R(ed.z), R(ed.w), dC, dD, ic, id, cnt, it, R(D.ks_distance), &s_dyn_it, sc);
                                    else k += fold_edge<EX, R>(pa, pc, mA, mC, R(-ed.z), R(ed.w), dA, dC, ia, ic, cnt, it, R(D.ks_distance), &s_dyn_it, sc);
                                }
                            }
                            if (k) {
                                const R terms = R(ktet > 1 ? ktet : 1);
                                if constexpr (S::kFixed) {
                                    if (abs_sum(dA) < wd.bound * terms && abs_sum(dB) < wd.bound * terms &&
                                        abs_sum(dC) < wd.bound * terms && abs_sum(dD) < wd.bound * terms) {
                                        acc_add<S>(acc, 3 * ia, dA.x); acc_add<S>(acc, 3 * ia + 1, dA.y); acc_add<S>(acc, 3 * ia + 2, dA.z);
                                        acc_add<S>(acc, 3 * ib, dB.x); acc_add<S>(acc, 3 * ib + 1, dB.y); acc_add<S>(acc, 3 * ib + 2, dB.z);
                                        acc_add<S>(acc, 3 * ic, dC.x); acc_add<S>(acc, 3 * ic + 1, dC.y); acc_add<S>(acc, 3 * ic + 2, dC.z);
                                        acc_add<S>(acc, 3 * id, dD.x); acc_add<S>(acc, 3 * id + 1, dD.y); acc_add<S>(acc, 3 * id + 2, dD.z);
                                    } else {
                                        add3s<S>(acc, ia, dA, bad, wd, terms); add3s<S>(acc, ib, dB, bad, wd, terms);
                                        add3s<S>(acc, ic, dC, bad, wd, terms); add3s<S>(acc, id, dD, bad, wd, terms);
                                    }
                                } else {
                                    add3s<S>(acc, ia, dA, bad, wd, terms); add3s<S>(acc, ib, dB, bad, wd, terms);
                                    add3s<S>(acc, ic, dC, bad, wd, terms); add3s<S>(acc, id, dD, bad, wd, terms);
                                }
                            }
                            if (skip) {
                                atomicSub(cnt + ia, skip); atomicSub(cnt + ib, skip);
                                atomicSub(cnt + ic, skip); atomicSub(cnt + id, skip);
                                s_dyn_it = it;
                            }
                        }
                    }
                    // ---- edge constraints: distance (integrator.py:65-109), XPBD (:191-240) ----
                    if (fl & (FFSRL_DISTANCE | FFSRL_DISTANCE_XPBD)) {
                        for (int e = tid; e < ne; e += BLOCK) {
                            const int ge = E.e0 + e;
                            const unsigned ix = __ldg(D.edge_idx + ge);
                            const int ia = ix & 0xffff, ib = ix >> 16;
                            const float2 la = __ldg(D.edge_la + ge);
                            const R active = R(la.y), L0 = R(la.x);
                            if (active == R(0) || L0 < R(BEPS)) continue;
                            const P PA = xp[ia], PB = xp[ib];
                            R mA = PA.w, mB = PB.w;
                            R w = mA + mB;
                            if (w < R(BEPS)) continue;  // never counted
                            const t3<R> dir = PO::pos(PB) - PO::pos(PA);
                            const R dd = dot(dir, dir);
                            R len, rl = R(0);
                            bool degenerate;
                            if constexpr (EX) {
                                len = sqrt(dd);
                                degenerate = len < R(BEPS);
                            } else {
                                degenerate = dd < R(BEPS * BEPS);  // length below FLOAT_EPSILON
                                rl = rsqrt_(dd);
                                len = dd * rl;
                            }
                            if (degenerate) {
                                const int skip = ((fl & FFSRL_DISTANCE) ? 1 : 0) + ((fl & FFSRL_DISTANCE_XPBD) ? 1 : 0);
                                atomicSub(cnt + ia, skip); atomicSub(cnt + ib, skip);
                                s_dyn_it = it;
                                continue;
                            }
                            const R C = len - L0;
                            t3<R> dA = T3<R>(0, 0, 0), dB = dA;
                            if (fl & FFSRL_DISTANCE) {
                                if constexpr (EX) {
                                    const t3<R> d = -C * (dir / len) * R(D.ks_distance) * active / w;
                                    dA = -((d * mA) * sc); dB = (d * mB) * sc;
                                } else {
                                    t3<R> d = dir * (-C * rl * R(D.ks_distance) * active * rcp(w));
                                    dA = -((d * mA) * sc); dB = (d * mB) * sc;
                                }
                            }
                            if (fl & FFSRL_DISTANCE_XPBD) {
                                R alpha = R(D.a_dist);
                                const int oe = E.me0 + __ldg(D.edge_orig + ge);
                                R lam = R(D.edge_lambda[oe]);
                                R dl = -(C + alpha * lam) / (w + alpha);
                                D.edge_lambda[oe] = float(lam + dl);
                                t3<R> d;
                                if constexpr (EX) d = dl * (dir / len);
                                else d = dir * (dl * rl);
                                dA = dA - (d * mA) * sc; dB = dB + (d * mB) * sc;
                            }
                            add3s<S>(acc, ia, dA, bad, wd, R(1)); add3s<S>(acc, ib, dB, bad, wd, R(1));
                        }
                    }
                    __syncthreads();
                    // ---- applyConstraints + dragConstraintsDO ----
                    const bool restore = s_dyn_it == it;
                    const bool wide_on = S::kFixed && s_wide_c[it & 1] != 0;
                    // for this iteration's contact phase (the previous one's reads are behind the
                    // barrier that ended it), and the next iteration's constraint phase
                    if (tid == 0) { s_any_contact = 0; s_near_n = 0; s_wide_k = 0; s_wide_c[(it + 1) & 1] = 0; }
                    for (int i = tid; i < nv; i += BLOCK) {
                        int c = cnt[i];
                        P q = xp[i];
                        t3<R> x = PO::pos(q);
                        long long pe[3];
                        const long long* extra = nullptr;
                        if (has_conn && D.conn_vert[E.v0 + i]) {
                            // the connector corrections of the previous iteration (or step) join
                            // this apply, as the reference's persistent dP does
                            const long long g = (long long)E.v0 + i;
                            c += D.pcnt[g];
                            pe[0] = D.pend[3 * g]; pe[1] = D.pend[3 * g + 1]; pe[2] = D.pend[3 * g + 2];
                            extra = pe;
                            D.pcnt[g] = 0;
                            D.pend[3 * g] = 0; D.pend[3 * g + 1] = 0; D.pend[3 * g + 2] = 0;
                        }
                        if (c > 0) {
                            const t3<R> s = take3<S>(acc, i, wide_on, wd, inv_sc, extra);
                            if constexpr (EX) {
                                const R n = R(c);
                                x = x + T3<R>(s.x / n, s.y / n, s.z / n);
                            } else {
                                const R rN = rcp(R(c));
                                x = x + T3<R>(s.x * rN, s.y * rN, s.z * rN);
                            }
                        }
                        if (restore) cnt[i] = __ldg(D.cnt0 + E.v0 + i);
                        if ((fl & FFSRL_DRAG) && s_any_drag && ((dbits[i >> 5] >> (i & 31)) & 1u)) {
                            R dr = R(__ldg(D.drag + E.v0 + i));
                            t3<R> dir = x - tool.drag_tip;
                            R len = length(dir);
                            if (!(len < R(BEPS))) x = x - len * normalize(dir) * dr * R(D.ks_drag) / R(2);
                        }
                        xp[i] = PO::make(x, q.w);
                    }
                    __syncthreads();
                    // ---- triToPointDistanceConstraintsDO (integrator.py:300-353): corrections for the
                    // next apply, from the positions after the grasp (before the contact) ----
                    if constexpr (S::kFixed) {
                        if (has_conn && E.nc > 0) {
                            for (int k = tid; k < E.nc; k += BLOCK) {
                                const uint2 ci = __ldg(D.conn_idx + E.c0 + k);
                                const float4 cb = __ldg(D.conn_bar + E.c0 + k);
                                const int v = ci.x & 0xffff, ta = ci.x >> 16, tb = ci.y & 0xffff, tc = ci.y >> 16;
                                const t3<R> bar = T3<R>(R(cb.x), R(cb.y), R(cb.z));
                                const t3<R> centre = PO::pos(xp[ta]) * bar.x + PO::pos(xp[tb]) * bar.y + PO::pos(xp[tc]) * bar.z;
                                const t3<R> dir = PO::pos(xp[v]) - centre;
                                const R len = length(dir);
                                if (len < R(BEPS)) continue;
                                const R wp = R(D.conn_w), wt = R(1) - wp;
                                const R Cc = len - R(cb.w) * R(D.conn_mul);
                                const R sden = wp + wt * (bar.x * bar.x + bar.y * bar.y + bar.z * bar.z);
                                const t3<R> delta = (Cc / sden) * (dir / len) * R(D.conn_ks);
                                const t3<R> part[4] = {-(delta * wp), delta * wt * bar.x, delta * wt * bar.y, delta * wt * bar.z};
                                const int vid[4] = {v, ta, tb, tc};
                                for (int q = 0; q < 4; ++q) {
                                    const t3<R> s = part[q] * sc;
                                    const R cs[3] = {s.x, s.y, s.z};
                                    for (int j = 0; j < 3; ++j) {
                                        if (!(fabsf(cs[j]) < kWideLimit)) { bad = true; continue; }
                                        atomicAdd(reinterpret_cast<unsigned long long*>(D.pend) + 3 * ((long long)E.v0 + vid[q]) + j,
                                                  (unsigned long long)__float2ll_rn(cs[j]));
                                    }
                                    atomicAdd(D.pcnt + E.v0 + vid[q], 1);
                                }
                            }
                        }
                    }
                    // ---- collideLaparoscopeDO (integrator.py:981-1050), positions as of phase start ----
                    // A scan tests every surface triangle's box against the capsules' boxes (their
                    // union first) and lists the near ones; the block then solves the listed
                    // triangles, one per thread, so the few contacts do not serialise a warp.
                    if ((fl & FFSRL_COLLIDE) && nf > 0) {
                        const R ks = R(D.ks_contact);
                        auto contact = [&](int a, int b, int c, const P& PA, const P& PB, const P& PC, unsigned near) {
                            const t3<R> pA = PO::pos(PA), pB = PO::pos(PB), pC = PO::pos(PC);
                            t3<R> centre = (pA + pB + pC) * R(0.3333f);
                            t3<R> n = normalize(cross(pB - pA, pC - pA));
                            t3<R> tA = T3<R>(0, 0, 0), tB = tA, tC = tA;
                            R tl = R(0);
                            for (int i = 0; i < 3; ++i) {
                                if (!((near >> i) & 1u)) continue;
                                t3<R> rA = T3<R>(0, 0, 0), rB = rA, rC = rA;
                                capsule_response(tool.tip[i], tool.base[i], tool.radius[i], n, centre, pA, pB, pC, ks, rA,
                                                 rB, rC);
                                tA = tA + rA; tB = tB + rB; tC = tC + rC;
                                tl = tl + length(rA) + length(rB) + length(rC);
                            }
                            if (tl > R(0)) atomicAdd(&s_incol, 1);
                            if (!(tl > R(0)) && !isnan(tl)) return;  // every response is zero
                            s_any_contact = 1;
                            if (PA.w > R(0)) add3s<S>(acc, a, tA * sc, bad, wk, R(1));
                            if (PB.w > R(0)) add3s<S>(acc, b, tB * sc, bad, wk, R(1));
                            if (PC.w > R(0)) add3s<S>(acc, c, tC * sc, bad, wk, R(1));
                        };
                        for (int f = tid; f < nf; f += BLOCK) {
                            const uint2 tr = tri_s ? tri_s[f] : __ldg(D.tri_idx + (long long)E.f0 + f);
                            if ((tr.y >> 16) == 1u) continue;
                            const int a = tr.x & 0xffff, b = tr.x >> 16, c = tr.y & 0xffff;
                            const P PA = xp[a], PB = xp[b], PC = xp[c];
                            const t3<R> lo = T3<R>(rmin(PA.x, rmin(PB.x, PC.x)), rmin(PA.y, rmin(PB.y, PC.y)),
                                                   rmin(PA.z, rmin(PB.z, PC.z)));
                            const t3<R> hi = T3<R>(rmax(PA.x, rmax(PB.x, PC.x)), rmax(PA.y, rmax(PB.y, PC.y)),
                                                   rmax(PA.z, rmax(PB.z, PC.z)));
                            if (lo.x > tool.uhi.x || lo.y > tool.uhi.y || lo.z > tool.uhi.z || hi.x < tool.ulo.x ||
                                hi.y < tool.ulo.y || hi.z < tool.ulo.z)
                                continue;
                            unsigned near = 0;
                            for (int i = 0; i < 3; ++i) {
                                bool apart = lo.x > tool.bhi[i].x || lo.y > tool.bhi[i].y || lo.z > tool.bhi[i].z ||
                                             hi.x < tool.blo[i].x || hi.y < tool.blo[i].y || hi.z < tool.blo[i].z;
                                if (!apart) near |= 1u << i;
                            }
                            if (!near) continue;
                            const int k = atomicAdd(&s_near_n, 1);
                            if (k < kNearCap) s_near[k] = ((unsigned)f << 3) | near;
                            else contact(a, b, c, PA, PB, PC, near);
                        }
                        __syncthreads();
                        const int nnear = min(s_near_n, kNearCap);  // the same for every thread
                        if (nnear > 0) {
                            for (int k = tid; k < nnear; k += BLOCK) {
                                const unsigned w = s_near[k];
                                const uint2 tr = tri_s ? tri_s[w >> 3] : __ldg(D.tri_idx + (long long)E.f0 + (w >> 3));
                                const int a = tr.x & 0xffff, b = tr.x >> 16, c = tr.y & 0xffff;
                                contact(a, b, c, xp[a], xp[b], xp[c], w & 7u);
                            }
                            __syncthreads();
                        }
                        if (s_any_contact) {
                            const bool cwide = S::kFixed && s_wide_k != 0;
                            for (int i = tid; i < nv; i += BLOCK) {
                                P q = xp[i];
                                const t3<R> d = take3<S>(acc, i, cwide, wk, inv_sc, nullptr);
                                xp[i] = PO::make(PO::pos(q) - d, q.w);
                            }
                            __syncthreads();
                        }
                    }
                }
                // ---- bounds (integrator.py:12-21) + PBDStep (:23-38) ----
                for (int i = tid; i < nv; i += BLOCK) {
                    P q = xp[i];
                    t3<R> p = PO::pos(q);
                    if (p.y < R(D.ground)) p.y = R(D.ground);
                    t3<R> x = ldgen3(D.vertex, E.v0 + i);
                    t3<R> v = (p - x) * (R(1) / dt);
                    stg3(D.vertex, E.v0 + i, p);
                    stg3(D.velocity, E.v0 + i, v);
                    xp[i] = PO::make(p, q.w);
                    bad |= !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z));
                }
                __syncthreads();
            }
        }
        for (int i = tid; i < nv; i += BLOCK) stg3(D.predicted, E.v0 + i, PO::pos(xp[i]));
        if (bad) s_bad = 1;
        __syncthreads();
        if (tid == 0) {
            if (s_incol) atomicAdd(D.in_collision + env, s_incol);
            D.env_status[env] = s_bad ? FFSRL_ERR_NONFINITE : FFSRL_OK;
        }
        __syncthreads();
    }
}

typedef void (*kern_f)(const Dev<float>, const int*, int, int*, int, unsigned char*, long long, int, int, int);
typedef void (*kern_d)(const Dev<double>, const int*, int, int*, int, unsigned char*, long long, int, int, int);

}  // namespace bk

// Kernel selection per unit.  prefetch 0: none, 1: L1 prefetch of the next record,
// 2: the next record held in registers (PIPE instantiations only).  A null result means
// no instantiation for that combination.
bk::kern_f pick_fast_fixed(int block, int mode, int prefetch, unsigned flags);       // batched.cu
bk::kern_f pick_ref_fixed(int block, int mode, int prefetch, unsigned flags);        // batched_ref.cu
bk::kern_f pick_ref_study(int accumulation, int block, int mode);                     // batched_study.cu
bk::kern_d pick_ref_f64(int block, int mode);                                         // batched_study.cu

}  // namespace ffsrl
