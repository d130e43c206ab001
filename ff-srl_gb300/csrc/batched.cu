// batched.cu -- env-resident batched step.
//
// One thread block owns one environment at a time and runs every substep and
// iteration of the step for it without leaving the SM: the env's predicted positions
// (with the inverse mass in .w) and its per-vertex correction accumulators live in
// shared memory, the read-only constraint tables stream from L2/HBM in coalesced
// structure-of-arrays records with 16-bit env-local vertex ids.  Blocks are persistent
// and take environments from a largest-first work list through an atomic counter, so
// meshes of uneven size share the GPU in one launch per size class.
//
// Semantics are SimIntegratorDO.stepModel's (FF_SRL/FF_SRL/integrator.py:1640-1741),
// Jacobi iteration unchanged: all constraint projections of an iteration read the same
// positions, their corrections are summed per vertex and divided by the number of
// contributing constraints (applyConstraints, integrator.py:946-960), then the grasp
// (dragConstraintsDO) and the instrument contact (collideLaparoscopeDO).
//
// Accumulation is deterministic: in float32 runs each correction component is rounded
// once to a 32-bit fixed-point integer and summed with native shared-memory integer
// atomics, which are associative, so the sum does not depend on thread order and an
// environment gives the same bits alone or in any batch.  The scale 2^k is chosen per
// model so that one unit is about a quarter of a float ulp of the largest coordinate
// (the position update itself rounds to an ulp); a contribution too large for the
// per-vertex sum to stay in range flags the environment as diverged.  The number of contributions per vertex
// is precomputed when the plan is built (a constraint only skips at run time on
// degenerate geometry, which then decrements it), so no count atomics are needed.
// Constraint records are ordered by a greedy vertex colouring within each environment so
// that the 32 lanes of a warp update distinct vertices.  The float64 build of the same
// kernel (used for the precision report) sums in double.
#include <cuda_runtime.h>
#include <cstdint>
#include <climits>
#include <vector>
#include <algorithm>
#include <numeric>
#include <cstring>
#include <string>
#include <cmath>
#include <unordered_map>
#include "ffsrl_internal.h"

namespace ffsrl {
namespace {

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
// Reciprocal and reciprocal square root: one hardware approximation each in float32
// (PTX rcp.approx / rsqrt.approx, about 1 ulp), exact division and sqrt in float64
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

// per-precision storage: predicted position + inverse mass, accumulator word
template <class R> struct Store;
struct Fixed { float scale, inv, bound; };

template <> struct Store<float> {
    typedef float4 P;
    typedef unsigned int A;
    __device__ static t3<float> pos(const P& p) { return T3<float>(p.x, p.y, p.z); }
    __device__ static P make(t3<float> v, float w) { return make_float4(v.x, v.y, v.z, w); }
    // callers have checked the range (in_range) before adding
    __device__ static void add(A* a, float v, const Fixed& fx) {
        atomicAdd(a, (unsigned)__float2int_rn(v * fx.scale));
    }
    // true when every |component| is below the per-term bound; the sum of magnitudes
    // also carries NaN and infinity into the test
    __device__ static bool in_range(float sum_abs, const Fixed& fx) { return sum_abs * fx.scale < fx.bound; }
    // the tet path forms its corrections already multiplied by the power-of-two scale
    // (exact), so only the conversion and the bound remain
    __device__ static float prescale(const Fixed& fx) { return fx.scale; }
    __device__ static void add_scaled(A* a, float v) { atomicAdd(a, (unsigned)__float2int_rn(v)); }
    __device__ static bool in_range_scaled(float sum_abs, const Fixed& fx, float terms) {
        return sum_abs < fx.bound * terms;
    }
    // a term that merges `terms` constraint contributions may use that many term bounds
    __device__ static bool in_range(float sum_abs, const Fixed& fx, float terms) {
        return sum_abs * fx.scale < fx.bound * terms;
    }
    __device__ static float get(A a, const Fixed& fx) { return __int2float_rn((int)a) * fx.inv; }
};
struct __align__(32) dpos { double x, y, z, w; };
template <> struct Store<double> {
    typedef dpos P;
    typedef double A;
    __device__ static t3<double> pos(const P& p) { return T3<double>(p.x, p.y, p.z); }
    __device__ static P make(t3<double> v, double w) { P r; r.x = v.x; r.y = v.y; r.z = v.z; r.w = w; return r; }
    __device__ static void add(A* a, double v, const Fixed&) { atomicAdd(a, v); }
    __device__ static bool in_range(double sum_abs, const Fixed&) { return sum_abs < 1.0e300; }
    __device__ static bool in_range(double sum_abs, const Fixed&, double) { return sum_abs < 1.0e300; }
    __device__ static double prescale(const Fixed&) { return 1.0; }
    __device__ static void add_scaled(A* a, double v) { atomicAdd(a, v); }
    __device__ static bool in_range_scaled(double sum_abs, const Fixed&, double) { return sum_abs < 1.0e300; }
    __device__ static double get(A a, const Fixed&) { return a; }
};

// v0/nv: the env's vertices in the model arrays; t0/e0/f0: its constraint tables, which
// envs with identical tables share; mt0/me0: its tets/edges in the model arrays (for the
// XPBD multipliers, which are per env)
struct EnvRec { int v0, nv, t0, nt, e0, ne, f0, nf, mt0, me0, c0, nc; };

template <class R> __device__ __forceinline__ R abs_sum(t3<R> d) { return fabs(d.x) + fabs(d.y) + fabs(d.z); }

// adds correction vectors to vertices' accumulators; a group whose magnitudes the
// fixed-point form cannot carry (non-finite or out of range) is dropped and raises `bad`
// so the env is reported diverged
template <class R> __device__ __forceinline__ void add3(typename Store<R>::A* acc, int i, t3<R> d, bool& bad,
                                                        const Fixed& fx) {
    if (!Store<R>::in_range(abs_sum(d), fx)) { bad = true; return; }
    Store<R>::add(acc + 3 * i, d.x, fx);
    Store<R>::add(acc + 3 * i + 1, d.y, fx);
    Store<R>::add(acc + 3 * i + 2, d.z, fx);
}
// The four corrections of one tet, already multiplied by the fixed-point scale; each
// vertex's term merges at least `terms` of the
// vertex's counted contributions (the tet's constraints), so it may use that many term
// bounds and the per-vertex sum still stays within int32.
template <class R> __device__ __forceinline__ void add3x4(typename Store<R>::A* acc, int ia, int ib, int ic, int id,
                                                          t3<R> dA, t3<R> dB, t3<R> dC, t3<R> dD, bool& bad,
                                                          const Fixed& fx, R terms) {
    typedef Store<R> S;
    if (!(S::in_range_scaled(abs_sum(dA), fx, terms) && S::in_range_scaled(abs_sum(dB), fx, terms) &&
          S::in_range_scaled(abs_sum(dC), fx, terms) && S::in_range_scaled(abs_sum(dD), fx, terms))) {
        bad = true;
        return;
    }
    S::add_scaled(acc + 3 * ia, dA.x); S::add_scaled(acc + 3 * ia + 1, dA.y); S::add_scaled(acc + 3 * ia + 2, dA.z);
    S::add_scaled(acc + 3 * ib, dB.x); S::add_scaled(acc + 3 * ib + 1, dB.y); S::add_scaled(acc + 3 * ib + 2, dB.z);
    S::add_scaled(acc + 3 * ic, dC.x); S::add_scaled(acc + 3 * ic + 1, dC.y); S::add_scaled(acc + 3 * ic + 2, dC.z);
    S::add_scaled(acc + 3 * id, dD.x); S::add_scaled(acc + 3 * id + 1, dD.y); S::add_scaled(acc + 3 * id + 2, dD.z);
}

template <class R> struct Dev {
    const EnvRec* env;
    const uint2* tet_idx;      // 4 x u16 local ids
    const float2* tet_va;      // (|V0|, active)
    const float4* nh0;         // Neo-Hookean: M = Dm^-1 Dm^-T entries (00, 01, 02, 11)
    const float4* nh1;         // (M12, M22, det Dm^-1, 1/|V0|)
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
    int fold;                  // distance constraints folded into the tet records
    const uint2* conn_idx;     // connectors: (point | triangle a << 16, b | c << 16), env-local ids
    const float4* conn_bar;    // (barycentric 0, 1, 2, rest distance)
    const unsigned char* conn_vert;  // per vertex (global id): 1 when a connector holds it
    int* pend;                 // [3V] connector corrections waiting for the next apply (fixed point)
    int* pcnt;                 // [V] their counts
    float conn_w, conn_ks, conn_mul;  // mass weight ratio, kS, rest length multiplier
    const int* tet_orig;       // env-local model tet id of each (colour-ordered) record, for XPBD lambdas
    const int* edge_orig;      // env-local model edge id of each record
    Fixed fx;
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

// One distance constraint between two of a tet's vertices, added to the tet's corrections
// (u gets -d m_u, v gets +d m_v), multiplied by the fixed-point scale `sc`.  Returns 1 when it contributed.  A degenerate length
// decrements the two static counts and records the iteration in *dyn_it.
template <class R> __device__ __forceinline__ int fold_edge(t3<R> pu, t3<R> pv, R mu, R mv, R L0, R active,
                                                            t3<R>& du, t3<R>& dv, int iu, int iv, int* cnt,
                                                            int it, R ks, int* dyn_it, R sc) {
    const R w = mu + mv;
    if (w < R(BEPS)) return 0;  // never counted
    const t3<R> dir = pv - pu;
    const R dd = dot(dir, dir);
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
template <class R> __host__ __device__ size_t smem_bytes(int mode, int max_nv) {
    size_t P = sizeof(typename Store<R>::P), A = sizeof(typename Store<R>::A);
    size_t bits = 4 * (size_t)((max_nv + 31) / 32 + 1);
    if (mode == 0) return (P + 3 * A + 4) * (size_t)max_nv + bits;
    if (mode == 1) return P * (size_t)max_nv + bits;
    return bits;
}

// MODE 0: positions and accumulators in shared memory.  MODE 1: positions in shared
// memory, accumulators in the block's global scratch.  MODE 2: both in global scratch.
// PIPE: the tet loop holds the thread's next tet record in registers, loaded while the
// current one is solved (for block sizes that leave the registers for it).
// FL: the constraint selection fixed at compile time (0: read from the parameters); the
// liver set (volume, distance, Neo-Hookean, grasp, contact) has its own instantiations.
constexpr unsigned kLiverFlags = FFSRL_VOLUME | FFSRL_DISTANCE | FFSRL_NEOHOOKEAN | FFSRL_DRAG | FFSRL_COLLIDE;

template <class R, int BLOCK, int MODE, bool PIPE = false, unsigned FL = 0>
__global__ void __launch_bounds__(BLOCK, (BLOCK <= 256 ? 768 / BLOCK : 1)) k_batched(const Dev<R> D, const int* __restrict__ work, int nwork,
                                                   int* counter, int nsteps, unsigned char* scratch,
                                                   long long scratch_stride, int max_nv, int prefetch,
                                                   int tri_cap) {
    typedef Store<R> S;
    typedef typename S::P P;
    typedef typename S::A A;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_work;
    __shared__ int s_incol;
    __shared__ int s_bad;
    __shared__ int s_any_contact;
    __shared__ int s_any_drag;
    __shared__ int s_dyn_it;  // iteration in which a constraint skipped on degenerate geometry
    __shared__ int s_near_n;
    __shared__ unsigned s_near[kNearCap];
    __shared__ ToolShared<R> tool;

    unsigned char* gbase = scratch + (long long)blockIdx.x * scratch_stride;
    const int tid = threadIdx.x;
    const R dt = R(D.dt);
    const unsigned fl = FL ? FL : D.flags;
    const bool has_conn = (fl & FFSRL_CONNECTORS) && D.conn_idx != nullptr;
    const Fixed fx = D.fx;
    const R sc = S::prescale(fx);  // power of two: scaling a product by it is exact
    // Neo-Hookean constants, hoisted with the reference's association order:
    // C offset invDev/invVol, and compliance/dT/dT (the per-tet /V0 stays per tet)
    const R nh_off = (R(1) / R(D.dev_c)) / (R(1) / R(D.vol_c));
    const R nh_uH = R(D.vol_c) / dt / dt;
    const R nh_uD = R(D.dev_c) / dt / dt;

    for (;;) {
        // the per-env flags are cleared before the barrier: after it, any warp may set them
        // (the grasp bits below set s_any_drag from every warp)
        if (tid == 0) {
            s_work = atomicAdd(counter, 1);
            s_incol = 0; s_bad = 0; s_any_drag = 0; s_dyn_it = -1;
        }
        __syncthreads();
        const int w = s_work;
        if (w >= nwork) return;
        const int env = work[w];
        const EnvRec E = D.env[env];
        const int nv = E.nv, nt = E.nt, ne = E.ne, nf = E.nf;

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
            tri_s = reinterpret_cast<uint2*>(smem + ((smem_bytes<R>(MODE, max_nv) + 7) & ~(size_t)7));
            for (int f = tid; f < nf; f += BLOCK) tri_s[f] = __ldg(D.tri_idx + (long long)E.f0 + f);
        }
        // inverse masses ride in .w for the whole step
        for (int i = tid; i < nv; i += BLOCK) {
            t3<R> x = ldgen3(D.vertex, E.v0 + i);
            xp[i] = S::make(x, R(__ldg(D.inv_mass + E.v0 + i)));
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
                    xp[i] = S::make(x + v * dt, inv);
                }
                if (fl & FFSRL_VOLUME_XPBD)
                    for (int t = tid; t < nt; t += BLOCK) D.tet_lambda[E.mt0 + t] = 0.0f;
                if (fl & FFSRL_DISTANCE_XPBD)
                    for (int e = tid; e < ne; e += BLOCK) D.edge_lambda[E.me0 + e] = 0.0f;
                __syncthreads();

                for (int it = 0; it < D.iterations; ++it) {
                    // ---- tet constraints: volume, XPBD volume, Neo-Hookean ----
                    if (fl & (FFSRL_VOLUME | FFSRL_VOLUME_XPBD | FFSRL_NEOHOOKEAN)) {
                        const bool nhf = (fl & FFSRL_NEOHOOKEAN) != 0;
                        uint2 ix_n = make_uint2(0u, 0u);
                        float2 va_n = make_float2(0.f, 0.f);
                        float4 n0_n = make_float4(0.f, 0.f, 0.f, 0.f), n1_n = n0_n, ed_n = n0_n;
                        if (PIPE && tid < nt) {
                            const int g0 = E.t0 + tid;
                            ix_n = __ldg(D.tet_idx + g0); va_n = __ldg(D.tet_va + g0);
                            if (nhf) { n0_n = __ldg(D.nh0 + g0); n1_n = __ldg(D.nh1 + g0); }
                            if (D.fold) ed_n = __ldg(D.tet_ed + g0);
                        }
                        for (int t = tid; t < nt; t += BLOCK) {
                            const int gt = E.t0 + t;
                            uint2 ix;
                            float2 va;
                            float4 n0, n1, ed;
                            if (PIPE) {
                                ix = ix_n; va = va_n; n0 = n0_n; n1 = n1_n; ed = ed_n;
                                if (t + BLOCK < nt) {  // the next record, in flight while this tet is solved
                                    const int gn = gt + BLOCK;
                                    ix_n = __ldg(D.tet_idx + gn); va_n = __ldg(D.tet_va + gn);
                                    if (nhf) { n0_n = __ldg(D.nh0 + gn); n1_n = __ldg(D.nh1 + gn); }
                                    if (D.fold) ed_n = __ldg(D.tet_ed + gn);
                                }
                            } else {
                                if (prefetch && t + BLOCK < nt) {  // this thread's next record, into L1
                                    const int gn = gt + BLOCK;
                                    prefetch_l1(D.tet_idx + gn);
                                    prefetch_l1(D.tet_va + gn);
                                    if (nhf) { prefetch_l1(D.nh0 + gn); prefetch_l1(D.nh1 + gn); }
                                    if (D.fold) prefetch_l1(D.tet_ed + gn);
                                }
                                // every record of the tet is requested up front, so its loads are in
                                // flight together
                                ix = __ldg(D.tet_idx + gt);
                                va = __ldg(D.tet_va + gt);
                                n0 = n1 = ed = make_float4(0.f, 0.f, 0.f, 0.f);
                                if (nhf) { n0 = __ldg(D.nh0 + gt); n1 = __ldg(D.nh1 + gt); }
                                if (D.fold) ed = __ldg(D.tet_ed + gt);
                            }
                            const int ia = ix.x & 0xffff, ib = ix.x >> 16, ic = ix.y & 0xffff, id = ix.y >> 16;
                            const P PA = xp[ia], PB = xp[ib], PC = xp[ic], PD = xp[id];
                            const t3<R> pa = S::pos(PA), pb = S::pos(PB), pc = S::pos(PC), pd = S::pos(PD);
                            const R mA = PA.w, mB = PB.w, mC = PC.w, mD = PD.w;
                            const t3<R> p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
                            t3<R> dA = T3<R>(0, 0, 0), dB = dA, dC = dA, dD = dA;
                            int k = 0;     // constraints that contributed
                            int skip = 0;  // statically counted constraints that skipped on degenerate geometry
                            const bool anym = mA != R(0) || mB != R(0) || mC != R(0) || mD != R(0);
                            // cofactor columns of Ds = [p1 p2 p3]: the volume gradient, and (times det Dm^-1) the
                            // Neo-Hookean hydrostatic gradient cof(F) Dm^-T = det(Dm^-1) cof(Ds)
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
                                            R C = R(va.x) - fabs(s6) * R(1.0 / 6.0);
                                            const R dl = -R(D.ks_volume) * active * C * rcp(wq) * sc;
                                            dA = q0 * dl * mA; dB = q1 * dl * mB; dC = q2 * dl * mC; dD = q3 * dl * mD;
                                            ++k;
                                        }
                                        if (fl & FFSRL_VOLUME_XPBD) {
                                            R alpha = R(D.a_vol);
                                            const int ot = E.mt0 + __ldg(D.tet_orig + gt);
                                            R lam = R(D.tet_lambda[ot]);
                                            R C = s6 / R(6) - R(__ldg(D.tet_vs + gt));
                                            R dl = -(C + alpha * lam) / (wq + alpha);
                                            D.tet_lambda[ot] = float(lam + dl);
                                            const R dls = dl * sc;
                                            dA = dA + q0 * dls * mA; dB = dB + q1 * dls * mB; dC = dC + q2 * dls * mC; dD = dD + q3 * dls * mD;
                                            ++k;
                                        }
                                    }
                                }
                            }
                            if (fl & FFSRL_NEOHOOKEAN) {
                                // neoHookeanConstraints (integrator.py:578-698) with F = Ds Dm^-1 written through
                                // M = Dm^-1 Dm^-T: |F|^2 = sum_ij (Ds^T Ds)_ij M_ij, F Dm^-T = Ds M, det F = det Ds det Dm^-1
                                const R m00 = R(n0.x), m01 = R(n0.y), m02 = R(n0.z), m11 = R(n0.w);
                                const R m12 = R(n1.x), m22 = R(n1.y), detD = R(n1.z), inv_rv = R(n1.w);
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
                            const int ktet = k;  // tet constraints merged into each vertex's term
                            if (D.fold) {
                                // distanceConstraints (integrator.py:65-109) of the edges this tet solves
                                if (ed.y != 0.0f) k += fold_edge<R>(pa, pb, mA, mB, R(ed.x), R(ed.y), dA, dB, ia, ib, cnt, it, R(D.ks_distance), &s_dyn_it, sc);
                                if (ed.w != 0.0f) {
                                    if (ed.z > 0.0f) k += fold_edge<R>(pc, pd, mC, mD, R(ed.z), R(ed.w), dC, dD, ic, id, cnt, it, R(D.ks_distance), &s_dyn_it, sc);
                                    else k += fold_edge<R>(pa, pc, mA, mC, R(-ed.z), R(ed.w), dA, dC, ia, ic, cnt, it, R(D.ks_distance), &s_dyn_it, sc);
                                }
                            }
                            if (k) add3x4<R>(acc, ia, ib, ic, id, dA, dB, dC, dD, bad, fx, R(ktet > 1 ? ktet : 1));
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
                            const t3<R> dir = S::pos(PB) - S::pos(PA);
                            const R dd = dot(dir, dir);
                            if (dd < R(BEPS * BEPS)) {  // length below FLOAT_EPSILON
                                const int skip = ((fl & FFSRL_DISTANCE) ? 1 : 0) + ((fl & FFSRL_DISTANCE_XPBD) ? 1 : 0);
                                atomicSub(cnt + ia, skip); atomicSub(cnt + ib, skip);
                                s_dyn_it = it;
                                continue;
                            }
                            const R rl = rsqrt_(dd);
                            const R C = dd * rl - L0;
                            t3<R> dA = T3<R>(0, 0, 0), dB = dA;
                            int k = 0;
                            if (fl & FFSRL_DISTANCE) {
                                t3<R> d = dir * (-C * rl * R(D.ks_distance) * active * rcp(w));
                                dA = -(d * mA); dB = d * mB;
                                ++k;
                            }
                            if (fl & FFSRL_DISTANCE_XPBD) {
                                R alpha = R(D.a_dist);
                                const int oe = E.me0 + __ldg(D.edge_orig + ge);
                                R lam = R(D.edge_lambda[oe]);
                                R dl = -(C + alpha * lam) / (w + alpha);
                                D.edge_lambda[oe] = float(lam + dl);
                                t3<R> d = dir * (dl * rl);
                                dA = dA - d * mA; dB = dB + d * mB;
                                ++k;
                            }
                            add3<R>(acc, ia, dA, bad, fx); add3<R>(acc, ib, dB, bad, fx);
                        }
                    }
                    __syncthreads();
                    // ---- applyConstraints + dragConstraintsDO ----
                    const bool restore = s_dyn_it == it;
                    if (tid == 0) { s_any_contact = 0; s_near_n = 0; }  // for this iteration's contact phase
                    for (int i = tid; i < nv; i += BLOCK) {
                        int c = cnt[i];
                        P q = xp[i];
                        t3<R> x = S::pos(q);
                        A s0 = acc[3 * i], s1 = acc[3 * i + 1], s2 = acc[3 * i + 2];
                        if (has_conn && D.conn_vert[E.v0 + i]) {
                            // the connector corrections of the previous iteration (or step) join
                            // this apply, as the reference's persistent dP does
                            const long long g = (long long)E.v0 + i;
                            c += D.pcnt[g];
                            s0 += A(D.pend[3 * g]); s1 += A(D.pend[3 * g + 1]); s2 += A(D.pend[3 * g + 2]);
                            D.pcnt[g] = 0;
                            D.pend[3 * g] = 0; D.pend[3 * g + 1] = 0; D.pend[3 * g + 2] = 0;
                        }
                        if (c > 0) {
                            const R rN = rcp(R(c));
                            x = x + T3<R>(S::get(s0, fx) * rN, S::get(s1, fx) * rN, S::get(s2, fx) * rN);
                            acc[3 * i] = A(0); acc[3 * i + 1] = A(0); acc[3 * i + 2] = A(0);
                        }
                        if (restore) cnt[i] = __ldg(D.cnt0 + E.v0 + i);
                        if ((fl & FFSRL_DRAG) && s_any_drag && ((dbits[i >> 5] >> (i & 31)) & 1u)) {
                            R dr = R(__ldg(D.drag + E.v0 + i));
                            t3<R> dir = x - tool.drag_tip;
                            R len = length(dir);
                            if (!(len < R(BEPS))) x = x - len * normalize(dir) * dr * R(D.ks_drag) / R(2);
                        }
                        xp[i] = S::make(x, q.w);
                    }
                    __syncthreads();
                    // ---- triToPointDistanceConstraintsDO (integrator.py:300-353): corrections for the
                    // next apply, from the positions after the grasp (before the contact) ----
                    if (has_conn && E.nc > 0) {
                        for (int k = tid; k < E.nc; k += BLOCK) {
                            const uint2 ci = __ldg(D.conn_idx + E.c0 + k);
                            const float4 cb = __ldg(D.conn_bar + E.c0 + k);
                            const int v = ci.x & 0xffff, ta = ci.x >> 16, tb = ci.y & 0xffff, tc = ci.y >> 16;
                            const t3<R> bar = T3<R>(R(cb.x), R(cb.y), R(cb.z));
                            const t3<R> centre = S::pos(xp[ta]) * bar.x + S::pos(xp[tb]) * bar.y + S::pos(xp[tc]) * bar.z;
                            const t3<R> dir = S::pos(xp[v]) - centre;
                            const R len = length(dir);
                            if (len < R(BEPS)) continue;
                            const R wp = R(D.conn_w), wt = R(1) - wp;
                            const R Cc = len - R(cb.w) * R(D.conn_mul);
                            const R sden = wp + wt * (bar.x * bar.x + bar.y * bar.y + bar.z * bar.z);
                            const t3<R> delta = (Cc / sden) * (dir / len) * R(D.conn_ks);
                            A* pend = reinterpret_cast<A*>(D.pend);
                            add3<R>(pend, E.v0 + v, -(delta * wp), bad, fx);
                            add3<R>(pend, E.v0 + ta, delta * wt * bar.x, bad, fx);
                            add3<R>(pend, E.v0 + tb, delta * wt * bar.y, bad, fx);
                            add3<R>(pend, E.v0 + tc, delta * wt * bar.z, bad, fx);
                            atomicAdd(D.pcnt + E.v0 + v, 1); atomicAdd(D.pcnt + E.v0 + ta, 1);
                            atomicAdd(D.pcnt + E.v0 + tb, 1); atomicAdd(D.pcnt + E.v0 + tc, 1);
                        }
                    }
                    // ---- collideLaparoscopeDO (integrator.py:981-1050), positions as of phase start ----
                    // A scan tests every surface triangle's box against the capsules' boxes (their
                    // union first) and lists the near ones; the block then solves the listed
                    // triangles, one per thread, so the few contacts do not serialise a warp.
                    if ((fl & FFSRL_COLLIDE) && nf > 0) {
                        const R ks = R(D.ks_contact);
                        auto contact = [&](int a, int b, int c, const P& PA, const P& PB, const P& PC, unsigned near) {
                            const t3<R> pA = S::pos(PA), pB = S::pos(PB), pC = S::pos(PC);
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
                            if (PA.w > R(0)) add3<R>(acc, a, tA, bad, fx);
                            if (PB.w > R(0)) add3<R>(acc, b, tB, bad, fx);
                            if (PC.w > R(0)) add3<R>(acc, c, tC, bad, fx);
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
                            for (int i = tid; i < nv; i += BLOCK) {
                                P q = xp[i];
                                t3<R> d = T3<R>(S::get(acc[3 * i], fx), S::get(acc[3 * i + 1], fx), S::get(acc[3 * i + 2], fx));
                                xp[i] = S::make(S::pos(q) - d, q.w);
                                acc[3 * i] = A(0); acc[3 * i + 1] = A(0); acc[3 * i + 2] = A(0);
                            }
                            __syncthreads();
                        }
                    }
                }
                // ---- bounds (integrator.py:12-21) + PBDStep (:23-38) ----
                for (int i = tid; i < nv; i += BLOCK) {
                    P q = xp[i];
                    t3<R> p = S::pos(q);
                    if (p.y < R(D.ground)) p.y = R(D.ground);
                    t3<R> x = ldgen3(D.vertex, E.v0 + i);
                    t3<R> v = (p - x) * (R(1) / dt);
                    stg3(D.vertex, E.v0 + i, p);
                    stg3(D.velocity, E.v0 + i, v);
                    xp[i] = S::make(p, q.w);
                    bad |= !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z));
                }
                __syncthreads();
            }
        }
        for (int i = tid; i < nv; i += BLOCK) stg3(D.predicted, E.v0 + i, S::pos(xp[i]));
        if (bad) s_bad = 1;
        __syncthreads();
        if (tid == 0) {
            if (s_incol) atomicAdd(D.in_collision + env, s_incol);
            D.env_status[env] = s_bad ? FFSRL_ERR_NONFINITE : FFSRL_OK;
        }
        __syncthreads();
    }
}

template <class R> size_t scratch_bytes(int mode, int max_nv) {
    size_t P = sizeof(typename Store<R>::P), A = sizeof(typename Store<R>::A);
    if (mode == 0) return 0;
    if (mode == 1) return (3 * A + 4) * (size_t)max_nv;
    return (P + 3 * A + 4) * (size_t)max_nv;
}

typedef void (*kern_f)(const Dev<float>, const int*, int, int*, int, unsigned char*, long long, int, int, int);
typedef void (*kern_d)(const Dev<double>, const int*, int, int*, int, unsigned char*, long long, int, int, int);

// prefetch 0: none, 1: L1 prefetch of the next record, 2: the next record held in
// registers (PIPE instantiations only)
kern_f pick_f(int block, int mode, int prefetch = 0, unsigned flags = 0) {
    if (flags == kLiverFlags && mode == 0 && prefetch != 2) {
        if (block == 256) return k_batched<float, 256, 0, false, kLiverFlags>;
        if (block == 512) return k_batched<float, 512, 0, false, kLiverFlags>;
        if (block == 640) return k_batched<float, 640, 0, false, kLiverFlags>;
        if (block == 768) return k_batched<float, 768, 0, false, kLiverFlags>;
        if (block == 1024) return k_batched<float, 1024, 0, false, kLiverFlags>;
    }
    if (prefetch == 2) {
        if (mode == 0 && block == 512) return k_batched<float, 512, 0, true>;
        if (mode == 0 && block == 640) return k_batched<float, 640, 0, true>;
        return nullptr;
    }
#define PK(B, M) if (block == B && mode == M) return k_batched<float, B, M>;
    PK(128, 0) PK(256, 0) PK(512, 0) PK(640, 0) PK(768, 0) PK(1024, 0)
    PK(256, 1) PK(512, 1) PK(1024, 1)
    PK(256, 2) PK(512, 2)
#undef PK
    return nullptr;
}
kern_d pick_d(int block, int mode) {
    if (block == 256 && mode == 0) return k_batched<double, 256, 0>;
    if (block == 256 && mode == 2) return k_batched<double, 256, 2>;
    return nullptr;
}

}  // namespace
}  // namespace ffsrl

using namespace ffsrl;

struct ffsrl_batch {
    int num_envs = 0;
    int precision = 32;
    int sm_count = 0, max_smem = 0;
    ffsrl_params params{};
    ffsrl_model dm{};  // device pointers of the model
    // device tables
    EnvRec* d_env = nullptr;
    uint2* d_tet_idx = nullptr; float2* d_tet_va = nullptr;
    float4* d_nh0 = nullptr; float4* d_nh1 = nullptr; float* d_tet_vs = nullptr; float4* d_tet_ed = nullptr;
    unsigned* d_edge_idx = nullptr; float2* d_edge_la = nullptr; uint2* d_tri_idx = nullptr;
    int* d_work = nullptr; int* d_counters = nullptr; int* d_status = nullptr;
    unsigned char* d_scratch = nullptr;
    double* d_state64 = nullptr;  // x, v, xp in double for precision 64
    int* d_cnt0 = nullptr;        // static per-vertex contribution counts
    int* d_tet_orig = nullptr;    // record -> model tet id
    int* d_edge_orig = nullptr;   // record -> model edge id
    uint2* d_conn_idx = nullptr; float4* d_conn_bar = nullptr; unsigned char* d_conn_vert = nullptr;
    int* d_pend = nullptr; int* d_pcnt = nullptr;  // pending connector corrections, kept between steps
    Fixed fx{1.0f, 1.0f, 1.0f};
    int64_t device_bytes = 0;
    size_t dyn_budget = 0;
    // classes
    struct Class {
        int mode, block, max_nv, grid, members;
        int prefetch = 0;  // L1 prefetch of the next tet record (autotuned)
        int tri_cap = 0;   // surface triangles kept in shared memory per env (0: read from L2)
        size_t smem, scratch_stride, scratch_offset;
        int work_offset, work_count;
    };
    std::vector<Class> classes;
    std::vector<int> env_class;
    std::vector<int> work_host;  // per class, largest first
    std::vector<int64_t> env_cost;
    // A lane is one in-flight launch sequence: its own class streams, work list, work
    // counters and scratch, so steps of disjoint env sets on different lanes can overlap.
    struct Lane {
        cudaEvent_t fork = nullptr, staged = nullptr;
        std::vector<cudaStream_t> streams;
        std::vector<cudaEvent_t> done;
        int* d_counters = nullptr;
        int* d_work_sub = nullptr;
        int* h_work_pinned = nullptr;
        bool staged_pending = false;
    };
    std::vector<Lane> lanes;
    size_t scratch_per_lane = 0;
};

namespace {

template <class T> int32_t dalloc(ffsrl_batch* b, T** p, size_t n) {
    if (n == 0) { *p = nullptr; return FFSRL_OK; }
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, "ffsrl_batch: cudaMalloc");
    b->device_bytes += (int64_t)(n * sizeof(T));
    return FFSRL_OK;
}
template <class T> int32_t upload(T* d, const std::vector<T>& h) {
    if (h.empty()) return FFSRL_OK;
    cudaError_t e = cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "ffsrl_batch: upload");
    return FFSRL_OK;
}

void free_batch(ffsrl_batch* b) {
    if (!b) return;
    cudaFree(b->d_env); cudaFree(b->d_tet_idx); cudaFree(b->d_tet_va); cudaFree(b->d_nh0); cudaFree(b->d_nh1); cudaFree(b->d_tet_ed);
    cudaFree(b->d_tet_vs); cudaFree(b->d_edge_idx); cudaFree(b->d_edge_la); cudaFree(b->d_tri_idx);
    cudaFree(b->d_work); cudaFree(b->d_status); cudaFree(b->d_scratch);
    cudaFree(b->d_state64); cudaFree(b->d_cnt0); cudaFree(b->d_tet_orig);
    cudaFree(b->d_edge_orig);
    cudaFree(b->d_conn_idx); cudaFree(b->d_conn_bar); cudaFree(b->d_conn_vert); cudaFree(b->d_pend); cudaFree(b->d_pcnt);
    for (auto& l : b->lanes) {
        for (auto s : l.streams) if (s) cudaStreamDestroy(s);
        for (auto e : l.done) if (e) cudaEventDestroy(e);
        if (l.fork) cudaEventDestroy(l.fork);
        if (l.staged) cudaEventDestroy(l.staged);
        cudaFree(l.d_counters);
        cudaFree(l.d_work_sub);
        if (l.h_work_pinned) cudaFreeHost(l.h_work_pinned);
    }
    delete b;
}

int default_block(int max_nv, int mode) {
    if (mode == 2) return 256;
    if (max_nv <= 256) return 128;
    if (max_nv <= 1024) return 256;
    if (max_nv <= 2560) return 512;
    return 1024;
}

template <class R> int32_t launch_class(ffsrl_batch* b, const ffsrl_batch::Class& c, const int* work, int nwork,
                                        int* counter, unsigned char* scratch, int nsteps, cudaStream_t s);

Dev<float> make_dev_f(ffsrl_batch* b) {
    Dev<float> D;
    const ffsrl_params& p = b->params;
    D.env = b->d_env; D.tet_idx = b->d_tet_idx; D.tet_va = b->d_tet_va; D.nh0 = b->d_nh0; D.nh1 = b->d_nh1;
    D.tet_vs = b->d_tet_vs; D.edge_idx = b->d_edge_idx; D.edge_la = b->d_edge_la;
    D.tri_idx = b->d_tri_idx;
    D.vertex = b->dm.vertex; D.velocity = b->dm.velocity; D.predicted = b->dm.predicted_vertex;
    D.inv_mass = b->dm.inverse_mass; D.drag = b->dm.active_drag_constraint;
    D.lap_base = b->dm.laparoscope_base; D.lap_tip = b->dm.laparoscope_tip; D.lap_radius = b->dm.laparoscope_radius;
    D.in_collision = b->dm.laparoscope_in_collision;
    D.tet_lambda = b->dm.tetrahedron_lambda; D.edge_lambda = b->dm.edge_lambda;
    D.env_status = b->d_status;
    D.cnt0 = b->d_cnt0; D.tet_orig = b->d_tet_orig; D.edge_orig = b->d_edge_orig; D.fx = b->fx;
    D.tet_ed = b->d_tet_ed; D.fold = b->d_tet_ed != nullptr;
    D.conn_idx = b->d_conn_idx; D.conn_bar = b->d_conn_bar; D.conn_vert = b->d_conn_vert;
    D.pend = b->d_pend; D.pcnt = b->d_pcnt;
    D.conn_w = p.connector_mass_weight_ratio; D.conn_ks = p.connector_ks; D.conn_mul = p.connector_rest_length_mul;
    D.flags = p.flags; D.substeps = p.substeps; D.iterations = p.iterations;
    D.dt = p.dt; D.gx = p.gravity[0]; D.gy = p.gravity[1]; D.gz = p.gravity[2];
    D.damping = p.velocity_dampening; D.ground = p.ground_level;
    D.ks_distance = p.ks_distance; D.ks_volume = p.ks_volume; D.ks_contact = p.ks_contact; D.ks_drag = p.ks_drag;
    D.vol_c = p.volume_compliance; D.dev_c = p.deviatoric_compliance;
    D.a_dist = (float)((double)p.distance_compliance / ((double)p.dt * (double)p.dt));
    D.a_vol = (float)((double)p.volume_compliance_xpbd / ((double)p.dt * (double)p.dt));
    return D;
}

template <> int32_t launch_class<float>(ffsrl_batch* b, const ffsrl_batch::Class& c, const int* work, int nwork,
                                        int* counter, unsigned char* scratch, int nsteps, cudaStream_t s) {
    kern_f k = pick_f(c.block, c.mode, c.prefetch, b->params.flags);
    if (!k) return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch: no kernel for block/mode");
    Dev<float> D = make_dev_f(b);
    int grid = std::min(c.grid, nwork);
    if (grid <= 0) return FFSRL_OK;
    k<<<grid, c.block, c.smem, s>>>(D, work, nwork, counter, nsteps, scratch + c.scratch_offset,
                                    (long long)c.scratch_stride, c.max_nv, c.prefetch == 1 ? 1 : 0, c.tri_cap);
    FFSRL_LAUNCH_CHECK("ffsrl_batch: step kernel");
    return FFSRL_OK;
}

template <> int32_t launch_class<double>(ffsrl_batch* b, const ffsrl_batch::Class& c, const int* work, int nwork,
                                         int* counter, unsigned char* scratch, int nsteps, cudaStream_t s) {
    kern_d k = pick_d(c.block, c.mode);
    if (!k) return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch: no float64 kernel for block/mode");
    Dev<float> F = make_dev_f(b);
    Dev<double> D;
    // same tables and parameters; state in the plan's double arrays
    D.env = F.env; D.tet_idx = F.tet_idx; D.tet_va = F.tet_va; D.nh0 = F.nh0; D.nh1 = F.nh1;
    D.tet_vs = F.tet_vs; D.edge_idx = F.edge_idx; D.edge_la = F.edge_la; D.tri_idx = F.tri_idx;
    int64_t V = b->dm.num_vertices;
    D.vertex = b->d_state64; D.velocity = b->d_state64 + 3 * V; D.predicted = b->d_state64 + 6 * V;
    D.inv_mass = F.inv_mass; D.drag = F.drag; D.lap_base = F.lap_base; D.lap_tip = F.lap_tip;
    D.lap_radius = F.lap_radius; D.in_collision = F.in_collision; D.tet_lambda = F.tet_lambda;
    D.edge_lambda = F.edge_lambda; D.env_status = F.env_status; D.flags = F.flags; D.substeps = F.substeps;
    D.cnt0 = F.cnt0; D.tet_orig = F.tet_orig; D.edge_orig = F.edge_orig; D.fx = F.fx;
    D.tet_ed = F.tet_ed; D.fold = F.fold;
    D.iterations = F.iterations; D.dt = F.dt; D.gx = F.gx; D.gy = F.gy; D.gz = F.gz; D.damping = F.damping;
    D.ground = F.ground; D.ks_distance = F.ks_distance; D.ks_volume = F.ks_volume; D.ks_contact = F.ks_contact;
    D.ks_drag = F.ks_drag; D.vol_c = F.vol_c; D.dev_c = F.dev_c; D.a_dist = F.a_dist; D.a_vol = F.a_vol;
    int grid = std::min(c.grid, nwork);
    if (grid <= 0) return FFSRL_OK;
    k<<<grid, c.block, c.smem, s>>>(D, work, nwork, counter, nsteps, scratch + c.scratch_offset,
                                    (long long)c.scratch_stride, c.max_nv, c.prefetch == 1 ? 1 : 0, c.tri_cap);
    FFSRL_LAUNCH_CHECK("ffsrl_batch: float64 step kernel");
    return FFSRL_OK;
}

int32_t run(ffsrl_batch* b, int lane, const std::vector<int>& counts, const int* d_work_base,
            const std::vector<int>& offsets, int nsteps, cudaStream_t s) {
    auto& L = b->lanes[lane];
    unsigned char* scratch = b->d_scratch ? b->d_scratch + (size_t)lane * b->scratch_per_lane : nullptr;
    FFSRL_CUDA_TRY(cudaMemsetAsync(L.d_counters, 0, sizeof(int) * b->classes.size(), s));
    FFSRL_CUDA_TRY(cudaEventRecord(L.fork, s));
    for (size_t ci = 0; ci < b->classes.size(); ++ci) {
        auto& c = b->classes[ci];
        cudaStream_t cs = L.streams[ci];
        FFSRL_CUDA_TRY(cudaStreamWaitEvent(cs, L.fork, 0));
        if (counts[ci] > 0) {
            int32_t st = b->precision == 64
                             ? launch_class<double>(b, c, d_work_base + offsets[ci], counts[ci], L.d_counters + ci,
                                                    scratch, nsteps, cs)
                             : launch_class<float>(b, c, d_work_base + offsets[ci], counts[ci], L.d_counters + ci,
                                                   scratch, nsteps, cs);
            if (st) return st;
        }
        FFSRL_CUDA_TRY(cudaEventRecord(L.done[ci], cs));
        FFSRL_CUDA_TRY(cudaStreamWaitEvent(s, L.done[ci], 0));
    }
    return FFSRL_OK;
}

// Regroups records (already ordered so that records of one colour, hence vertex-disjoint,
// are contiguous) into the 32-record chunks a warp processes together, choosing for each
// lane the candidate (within `window` records of the same key) whose vertices add the
// fewest shared-memory bank collisions: the atomics on vertex v's accumulator words hit
// bank (3v + component) mod 32, one per vertex per corner and warp; the 16-byte position
// loads are served eight lanes at a time, colliding on v mod 8.  Only the order changes;
// every record keeps its own data.
template <class VertFn, class KeyFn>
void bank_regroup(std::vector<int>& ord, int corners, VertFn vert, KeyFn key, int window = 64) {
    const size_t n = ord.size();
    std::vector<int> out;
    out.reserve(n);
    std::vector<char> taken(n, 0);  // by position in ord
    size_t head = 0;
    int aload[4][32], qload[4][8];
    while (out.size() < n) {
        std::memset(aload, 0, sizeof(aload));
        for (int j = 0; j < 32 && out.size() < n; ++j) {
            if ((j & 7) == 0) std::memset(qload, 0, sizeof(qload));
            while (taken[head]) ++head;
            const int k0 = key(ord[head]);
            size_t best = head;
            int best_cost = INT32_MAX, scanned = 0;
            for (size_t i = head; i < n && scanned < window; ++i) {
                if (taken[i]) continue;
                const int r = ord[i];
                if (key(r) != k0) break;
                ++scanned;
                int cost = 0;
                for (int c = 0; c < corners; ++c) {
                    const int v = vert(r, c);
                    cost += 3 * aload[c][v & 31] + 4 * qload[c][v & 7];
                }
                if (cost < best_cost) { best_cost = cost; best = i; if (!cost) break; }
            }
            taken[best] = 1;
            const int r = ord[best];
            out.push_back(r);
            for (int c = 0; c < corners; ++c) {
                const int v = vert(r, c);
                ++aload[c][v & 31];
                ++qload[c][v & 7];
            }
        }
    }
    ord.swap(out);
}

// Block size of a class: the instantiation, its shared-memory allowance and the grid
// from the runtime's occupancy calculator.
constexpr int kLanes = 2;

int32_t configure_class(ffsrl_batch* b, ffsrl_batch::Class& c, int block, size_t dyn_budget) {
    if (b->precision == 64) block = 256;
    if (c.mode == 1 && block < 256) block = 256;
    if (c.mode == 2 && block > 512) block = 512;
    const void* kfn = b->precision == 64 ? (const void*)pick_d(block, c.mode)
                                         : (const void*)pick_f(block, c.mode, c.prefetch, b->params.flags);
    if (!kfn) return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch: no kernel for block " + std::to_string(block) +
                                                     " in mode " + std::to_string(c.mode));
    if (c.smem > 48 * 1024) {
        // several classes may share one instantiation: allow the whole budget
        cudaError_t ea = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_budget);
        if (ea != cudaSuccess) return cuda_fail(ea, "ffsrl_batch: shared memory attribute");
    }
    int per_sm = 0;
    cudaError_t eo = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, block, c.smem);
    if (eo != cudaSuccess || per_sm <= 0)
        return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch: class does not fit on an SM (block " + std::to_string(block) +
                                               ", shared " + std::to_string(c.smem) + ")");
    c.block = block;
    c.grid = std::max(1, std::min({c.members, per_sm * b->sm_count, c.scratch_stride ? 8 * b->sm_count : INT32_MAX}));
    return FFSRL_OK;
}

}  // namespace

extern "C" int32_t ffsrl_batch_create(const ffsrl_model* hm, const ffsrl_model* dmod, const ffsrl_params* p,
                                      const ffsrl_batch_options* opts, ffsrl_batch** out) {
    if (!hm || !dmod || !p || !out) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: null argument");
    *out = nullptr;
    const int N = hm->num_envs;
    if (N <= 0 || !hm->env_vertex_start || !hm->env_tet_start || !hm->env_edge_start || !hm->env_tri_start)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: host env ranges required");
    int precision = 32;
    int block_override = 0;
    if (opts) {
        block_override = opts->block_threads;
        if (opts->reserved[0] == 64) precision = 64;
    }
    const bool conn = (p->flags & FFSRL_CONNECTORS) && hm->num_connectors > 0;
    if (conn && (precision == 64 || !hm->connector_vertex_id || !hm->connector_triangle_id ||
                 !hm->connector_tri_bar || !hm->connector_rest_dist))
        return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch_create: connectors need the float32 step and all four "
                                           "connector arrays");
    ffsrl_batch* b = new ffsrl_batch();
    b->num_envs = N;
    b->params = *p;
    b->dm = *dmod;
    b->precision = precision;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&b->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (b->sm_count <= 0 || b->max_smem <= 0) { free_batch(b); return fail(FFSRL_ERR_CUDA, "ffsrl_batch_create: no device"); }
    // the kernels' static shared memory (block-wide scalars and the instrument) comes off
    // the per-block opt-in limit; budget dynamic shared memory below that
    size_t static_smem = 0;
    {
        const void* probes[] = {(const void*)pick_f(1024, 0), (const void*)pick_f(512, 1), (const void*)pick_d(256, 0)};
        for (const void* k : probes) {
            cudaFuncAttributes fa;
            if (cudaFuncGetAttributes(&fa, k) == cudaSuccess) static_smem = std::max(static_smem, fa.sharedSizeBytes);
        }
    }
    const size_t dyn_budget = (size_t)b->max_smem > static_smem + 64 ? (size_t)b->max_smem - static_smem - 64 : 0;
    b->dyn_budget = dyn_budget;

    const int64_t V = hm->num_vertices, T = hm->num_tetrahedrons, E = hm->num_edges, F = hm->num_triangles;
    std::vector<EnvRec> env(N);
    std::vector<uint2> tet_idx(T);
    std::vector<float2> tet_va(T);
    std::vector<float4> nh0, nh1;
    std::vector<float> tet_vs;
    const bool nh = (p->flags & FFSRL_NEOHOOKEAN) != 0;
    const bool xv = (p->flags & FFSRL_VOLUME_XPBD) != 0;
    if (nh && !hm->tetrahedron_dm_inv) { free_batch(b); return fail(FFSRL_ERR_INVALID_ARGUMENT, "Neo-Hookean needs tetrahedron_dm_inv"); }
    if (xv && (!hm->xpbd_rest_volume || !dmod->tetrahedron_lambda)) { free_batch(b); return fail(FFSRL_ERR_INVALID_ARGUMENT, "XPBD volume needs xpbd_rest_volume and lambdas"); }
    if ((p->flags & FFSRL_DISTANCE_XPBD) && !dmod->edge_lambda) { free_batch(b); return fail(FFSRL_ERR_INVALID_ARGUMENT, "XPBD distance needs edge_lambda"); }
    if (nh) { nh0.resize(T); nh1.resize(T); }
    if (xv) tet_vs.resize(T);
    std::vector<unsigned> edge_idx(E);
    std::vector<float2> edge_la(E);
    std::vector<uint2> tri_idx(F);
    for (int e = 0; e < N; ++e) {
        EnvRec r{};
        r.v0 = hm->env_vertex_start[e]; r.nv = hm->env_vertex_start[e + 1] - r.v0;
        r.t0 = hm->env_tet_start[e]; r.nt = hm->env_tet_start[e + 1] - r.t0;
        r.e0 = hm->env_edge_start[e]; r.ne = hm->env_edge_start[e + 1] - r.e0;
        r.f0 = hm->env_tri_start[e]; r.nf = hm->env_tri_start[e + 1] - r.f0;
        if (r.nv < 0 || r.nt < 0 || r.ne < 0 || r.nf < 0 || r.nv > 65535) {
            free_batch(b);
            return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch_create: env " + std::to_string(e) +
                                                   " has a negative range or more than 65535 vertices");
        }
        env[e] = r;
        auto local = [&](int g, int& outv) -> bool {
            int l = g - r.v0;
            if (l < 0 || l >= r.nv) return false;
            outv = l;
            return true;
        };
        for (int t = r.t0; t < r.t0 + r.nt; ++t) {
            int l[4];
            for (int k = 0; k < 4; ++k)
                if (!local(hm->tetrahedron[4ll * t + k], l[k])) {
                    free_batch(b);
                    return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: tet " + std::to_string(t) + " leaves its env");
                }
            tet_idx[t] = make_uint2((unsigned)l[0] | ((unsigned)l[1] << 16), (unsigned)l[2] | ((unsigned)l[3] << 16));
            tet_va[t] = make_float2(hm->tetrahedron_rest_volume ? hm->tetrahedron_rest_volume[t] : 0.0f,
                                    hm->active_tetrahedron ? hm->active_tetrahedron[t] : 1.0f);
            if (nh) {
                // M = D D^T and det D of the stored D = Dm^-1 (row-major), in double
                const float* f = hm->tetrahedron_dm_inv + 9ll * t;
                double d[9];
                for (int k = 0; k < 9; ++k) d[k] = f[k];
                auto mm = [&](int i, int j) { return d[3 * i] * d[3 * j] + d[3 * i + 1] * d[3 * j + 1] + d[3 * i + 2] * d[3 * j + 2]; };
                double det = d[0] * (d[4] * d[8] - d[5] * d[7]) - d[1] * (d[3] * d[8] - d[5] * d[6]) +
                             d[2] * (d[3] * d[7] - d[4] * d[6]);
                nh0[t] = make_float4((float)mm(0, 0), (float)mm(0, 1), (float)mm(0, 2), (float)mm(1, 1));
                const double v0 = hm->tetrahedron_rest_volume ? (double)hm->tetrahedron_rest_volume[t] : 0.0;
                nh1[t] = make_float4((float)mm(1, 2), (float)mm(2, 2), (float)det, (float)(1.0 / (double)(float)v0));
            }
            if (xv) tet_vs[t] = hm->xpbd_rest_volume[t];
        }
        for (int k = r.e0; k < r.e0 + r.ne; ++k) {
            int a, c;
            if (!local(hm->edge[2ll * k], a) || !local(hm->edge[2ll * k + 1], c)) {
                free_batch(b);
                return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: edge " + std::to_string(k) + " leaves its env");
            }
            edge_idx[k] = (unsigned)a | ((unsigned)c << 16);
            edge_la[k] = make_float2(hm->edge_rest_length[k], hm->active_edge ? hm->active_edge[k] : 1.0f);
        }
        for (int f = r.f0; f < r.f0 + r.nf; ++f) {
            int a, c, d;
            if (!local(hm->triangle[3ll * f], a) || !local(hm->triangle[3ll * f + 1], c) ||
                !local(hm->triangle[3ll * f + 2], d)) {
                free_batch(b);
                return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: triangle " + std::to_string(f) + " leaves its env");
            }
            unsigned h = (hm->hole && hm->hole[f] == 1) ? 1u : 0u;
            tri_idx[f] = make_uint2((unsigned)a | ((unsigned)c << 16), (unsigned)d | (h << 16));
        }
    }

    // ---- envs with identical tables and masses: the folding and ordering below are
    // computed once per distinct env and copied to its duplicates ----
    std::vector<int> dup_of(N, -1);
    {
        auto fnv = [](uint64_t h, const void* p, size_t n) {
            const unsigned char* c = static_cast<const unsigned char*>(p);
            for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
            return h;
        };
        auto rng_eq = [](const auto& v, int o1, int o2, int n) {
            return n == 0 || v.empty() || std::memcmp(&v[o1], &v[o2], sizeof(v[0]) * (size_t)n) == 0;
        };
        auto same = [&](const EnvRec& a, const EnvRec& c) {
            return a.nv == c.nv && a.nt == c.nt && a.ne == c.ne && a.nf == c.nf &&
                   std::memcmp(hm->inverse_mass + a.v0, hm->inverse_mass + c.v0, sizeof(float) * (size_t)a.nv) == 0 &&
                   rng_eq(tet_idx, a.t0, c.t0, a.nt) && rng_eq(tet_va, a.t0, c.t0, a.nt) &&
                   rng_eq(nh0, a.t0, c.t0, a.nt) && rng_eq(nh1, a.t0, c.t0, a.nt) && rng_eq(tet_vs, a.t0, c.t0, a.nt) &&
                   rng_eq(edge_idx, a.e0, c.e0, a.ne) && rng_eq(edge_la, a.e0, c.e0, a.ne) &&
                   rng_eq(tri_idx, a.f0, c.f0, a.nf);
        };
        std::unordered_map<uint64_t, std::vector<int>> first;
        for (int e = 0; e < N; ++e) {
            const EnvRec& r = env[e];
            uint64_t h = fnv(1469598103934665603ull, &r.nv, sizeof(int));
            h = fnv(h, &r.nt, sizeof(int));
            h = fnv(h, &r.ne, sizeof(int));
            if (r.nt) h = fnv(h, &tet_idx[r.t0], sizeof(uint2) * (size_t)std::min(r.nt, 256));
            if (r.nv) h = fnv(h, hm->inverse_mass + r.v0, sizeof(float) * (size_t)std::min(r.nv, 256));
            for (int c : first[h])
                if (same(r, env[c])) { dup_of[e] = c; break; }
            if (dup_of[e] < 0) first[h].push_back(e);
        }
    }

    // ---- static contribution counts (the runtime skips only on degenerate geometry) ----
    const float feps = (float)BEPS;
    std::vector<int> cnt0(V, 0), tri_deg(V, 0);
    const uint32_t fl = p->flags;
    for (int64_t t = 0; t < T; ++t) {
        const int32_t* q = hm->tetrahedron + 4 * t;
        bool anym = false;
        for (int k = 0; k < 4; ++k) anym |= hm->inverse_mass[q[k]] != 0.0f;
        if (!anym) continue;
        bool act = tet_va[t].y == 1.0f;
        int k = ((fl & FFSRL_VOLUME) && act ? 1 : 0) + ((fl & FFSRL_VOLUME_XPBD) && act ? 1 : 0) +
                ((fl & FFSRL_NEOHOOKEAN) ? 1 : 0);
        for (int j = 0; j < 4; ++j) cnt0[q[j]] += k;
    }
    for (int64_t e = 0; e < E; ++e) {
        const int32_t* q = hm->edge + 2 * e;
        float w = hm->inverse_mass[q[0]] + hm->inverse_mass[q[1]];
        if (edge_la[e].y == 0.0f || edge_la[e].x < feps || w < feps) continue;
        int k = ((fl & FFSRL_DISTANCE) ? 1 : 0) + ((fl & FFSRL_DISTANCE_XPBD) ? 1 : 0);
        cnt0[q[0]] += k; cnt0[q[1]] += k;
    }
    for (int64_t f = 0; f < F; ++f)
        for (int k = 0; k < 3; ++k) tri_deg[hm->triangle[3 * f + k]] += 1;
    int max_terms = 1;
    // ---- connectors (triToPointDistanceConstraintsDO): each belongs to the env of its
    // point, and all four of its vertices must lie in that env ----
    std::vector<uint2> conn_idx;
    std::vector<float4> conn_bar;
    std::vector<unsigned char> conn_vert;
    if (conn) {
        const int64_t C = hm->num_connectors;
        std::vector<std::vector<int>> per(N);
        auto env_of = [&](int g) {
            int lo = 0, hi = N - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) / 2;
                if (hm->env_vertex_start[mid] <= g) lo = mid; else hi = mid - 1;
            }
            return lo;
        };
        for (int64_t c = 0; c < C; ++c) {
            const int g[4] = {hm->connector_vertex_id[c], hm->connector_triangle_id[3 * c],
                              hm->connector_triangle_id[3 * c + 1], hm->connector_triangle_id[3 * c + 2]};
            for (int k = 0; k < 4; ++k)
                if (g[k] < 0 || g[k] >= V) {
                    free_batch(b);
                    return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: connector vertex id out of range");
                }
            const int e = env_of(g[0]);
            for (int k = 1; k < 4; ++k)
                if (env_of(g[k]) != e) {
                    free_batch(b);
                    return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch_create: connector " + std::to_string(c) +
                                                           " joins two environments");
                }
            per[e].push_back((int)c);
        }
        conn_vert.assign(V, 0);
        for (int e = 0; e < N; ++e) {
            env[e].c0 = (int)conn_idx.size();
            env[e].nc = (int)per[e].size();
            const int v0 = env[e].v0;
            for (int c : per[e]) {
                const int g[4] = {hm->connector_vertex_id[c], hm->connector_triangle_id[3ll * c],
                                  hm->connector_triangle_id[3ll * c + 1], hm->connector_triangle_id[3ll * c + 2]};
                for (int k = 0; k < 4; ++k) conn_vert[g[k]] = 1;
                conn_idx.push_back(make_uint2((unsigned)(g[0] - v0) | ((unsigned)(g[1] - v0) << 16),
                                              (unsigned)(g[2] - v0) | ((unsigned)(g[3] - v0) << 16)));
                conn_bar.push_back(make_float4(hm->connector_tri_bar[3ll * c], hm->connector_tri_bar[3ll * c + 1],
                                               hm->connector_tri_bar[3ll * c + 2], hm->connector_rest_dist[c]));
            }
        }
        // a connector adds one term to each of its vertices' sums
        for (int64_t c = 0; c < C; ++c) {
            tri_deg[hm->connector_vertex_id[c]] += 1;
            for (int k = 0; k < 3; ++k) tri_deg[hm->connector_triangle_id[3 * c + k]] += 1;
        }
    }
    for (int64_t v = 0; v < V; ++v) max_terms = std::max(max_terms, cnt0[v] + tri_deg[v]);

    // ---- fixed-point scale: one unit ~ a quarter float ulp of the largest coordinate ----
    {
        double mx = 1e-30;
        for (int64_t i = 0; i < 3 * V; ++i) mx = std::max(mx, (double)std::fabs(hm->vertex[i]));
        int e2 = 0;
        std::frexp(mx, &e2);  // mx < 2^e2
        int k = 26 - e2;
        b->fx.scale = std::ldexp(1.0f, k);
        b->fx.inv = std::ldexp(1.0f, -k);
        // each term below 2^31 / (terms + 1): the per-vertex sum cannot leave int32
        b->fx.bound = std::ldexp(1.0f, 31) / (float)(max_terms + 1);
    }

    // ---- fold distance constraints into tets: each edge is solved by one tet that holds
    // both its vertices, inside that tet's thread, so its correction joins the tet's four
    // accumulator updates.  A tet takes at most two edges; its vertices are reordered by an
    // even permutation (same orientation, Neo-Hookean tables recomputed for the new order)
    // so that the edges sit at A-B, and C-D or A-C.  Edges no tet can take stay in the
    // edge loop.  Not with XPBD distance (per-edge multipliers), so edge records keep their
    // model order otherwise. ----
    std::vector<float4> tet_ed;
    std::vector<unsigned char> tet_cls(T, 0);  // 0 none, 1 A-B, 2 A-B + C-D, 3 A-B + A-C
    const bool fold = (fl & FFSRL_DISTANCE) && !(fl & FFSRL_DISTANCE_XPBD) &&
                      (fl & (FFSRL_VOLUME | FFSRL_VOLUME_XPBD | FFSRL_NEOHOOKEAN)) && T > 0 && E > 0;
    if (fold) {
        tet_ed.assign(T, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        std::vector<unsigned> n_edge_idx;
        std::vector<float2> n_edge_la;
        std::vector<int> adj_start, adj;
        std::vector<int> owned_n(T, 0), owned(2 * T, -1);
        for (int e = 0; e < N; ++e) {
            EnvRec& r = env[e];
            if (dup_of[e] >= 0) {
                const EnvRec& src = env[dup_of[e]];
                std::copy(tet_idx.begin() + src.t0, tet_idx.begin() + src.t0 + r.nt, tet_idx.begin() + r.t0);
                std::copy(tet_ed.begin() + src.t0, tet_ed.begin() + src.t0 + r.nt, tet_ed.begin() + r.t0);
                std::copy(tet_cls.begin() + src.t0, tet_cls.begin() + src.t0 + r.nt, tet_cls.begin() + r.t0);
                if (nh) {
                    std::copy(nh0.begin() + src.t0, nh0.begin() + src.t0 + r.nt, nh0.begin() + r.t0);
                    std::copy(nh1.begin() + src.t0, nh1.begin() + src.t0 + r.nt, nh1.begin() + r.t0);
                }
                const int e0 = (int)n_edge_idx.size();
                for (int k = 0; k < src.ne; ++k) {
                    const unsigned ix = n_edge_idx[src.e0 + k];
                    const float2 la = n_edge_la[src.e0 + k];
                    n_edge_idx.push_back(ix);
                    n_edge_la.push_back(la);
                }
                r.e0 = e0;
                r.ne = src.ne;
                continue;
            }
            // vertex -> incident tets of this env
            adj_start.assign(r.nv + 1, 0);
            for (int t = r.t0; t < r.t0 + r.nt; ++t) {
                uint2 ix = tet_idx[t];
                int l[4] = {(int)(ix.x & 0xffff), (int)(ix.x >> 16), (int)(ix.y & 0xffff), (int)(ix.y >> 16)};
                for (int k = 0; k < 4; ++k) adj_start[l[k] + 1]++;
            }
            for (int v = 0; v < r.nv; ++v) adj_start[v + 1] += adj_start[v];
            adj.assign(adj_start[r.nv], 0);
            {
                std::vector<int> fill(adj_start.begin(), adj_start.end() - 1);
                for (int t = r.t0; t < r.t0 + r.nt; ++t) {
                    uint2 ix = tet_idx[t];
                    int l[4] = {(int)(ix.x & 0xffff), (int)(ix.x >> 16), (int)(ix.y & 0xffff), (int)(ix.y >> 16)};
                    for (int k = 0; k < 4; ++k) adj[fill[l[k]]++] = t;
                }
            }
            const int ne_new0 = (int)n_edge_idx.size();
            for (int k = r.e0; k < r.e0 + r.ne; ++k) {
                const int a = edge_idx[k] & 0xffff, c = edge_idx[k] >> 16;
                const float2 la = edge_la[k];
                const float w = hm->inverse_mass[r.v0 + a] + hm->inverse_mass[r.v0 + c];
                if (la.y == 0.0f || la.x < feps || w < feps) continue;  // never contributes or counts
                int best = -1;
                for (int j = adj_start[a]; j < adj_start[a + 1]; ++j) {
                    const int t = adj[j];
                    if (owned_n[t] >= 2) continue;
                    uint2 ix = tet_idx[t];
                    int l[4] = {(int)(ix.x & 0xffff), (int)(ix.x >> 16), (int)(ix.y & 0xffff), (int)(ix.y >> 16)};
                    if (l[0] != c && l[1] != c && l[2] != c && l[3] != c) continue;
                    if (best < 0 || owned_n[t] < owned_n[best]) best = t;
                }
                if (best >= 0) {
                    owned[2 * best + owned_n[best]++] = k;
                } else {
                    n_edge_idx.push_back(edge_idx[k]);
                    n_edge_la.push_back(la);
                }
            }
            // reorder each owning tet and record its edges
            for (int t = r.t0; t < r.t0 + r.nt; ++t) {
                if (!owned_n[t]) continue;
                uint2 ix = tet_idx[t];
                int l[4] = {(int)(ix.x & 0xffff), (int)(ix.x >> 16), (int)(ix.y & 0xffff), (int)(ix.y >> 16)};
                auto pos = [&](int v) { for (int q = 0; q < 4; ++q) if (l[q] == v) return q; return -1; };
                const int k1 = owned[2 * t], k2 = owned_n[t] > 1 ? owned[2 * t + 1] : -1;
                const int i1 = pos(edge_idx[k1] & 0xffff), j1 = pos(edge_idx[k1] >> 16);
                int nw[4];
                int cls = 1;
                if (k2 < 0) {
                    nw[0] = i1; nw[1] = j1;
                    int o = 2;
                    for (int q = 0; q < 4; ++q) if (q != i1 && q != j1) nw[o++] = q;
                } else {
                    const int i2 = pos(edge_idx[k2] & 0xffff), j2 = pos(edge_idx[k2] >> 16);
                    if (i2 != i1 && i2 != j1 && j2 != i1 && j2 != j1) {  // opposite: A-B, C-D
                        nw[0] = i1; nw[1] = j1; nw[2] = i2; nw[3] = j2;
                        cls = 2;
                    } else {  // adjacent: the shared vertex is A, then B and C
                        const int sh = (i2 == i1 || j2 == i1) ? i1 : j1;
                        const int o1 = sh == i1 ? j1 : i1, o2 = i2 == sh ? j2 : i2;
                        nw[0] = sh; nw[1] = o1; nw[2] = o2;
                        for (int q = 0; q < 4; ++q) if (q != sh && q != o1 && q != o2) nw[3] = q;
                        cls = 3;
                    }
                }
                // make the permutation even by swapping the two entries that carry no
                // edge constraint of their own (C and D for one edge; for two edges the
                // swap of A-B's ends or of the second pair's ends keeps the pairs)
                int inv = 0;
                for (int x = 0; x < 4; ++x)
                    for (int y = x + 1; y < 4; ++y) inv += nw[x] > nw[y];
                if (inv & 1) {
                    if (cls == 1 || cls == 2) std::swap(nw[2], nw[3]);
                    else std::swap(nw[1], nw[2]);  // A-B and A-C trade places: edges follow below
                }
                int nl[4];
                for (int q = 0; q < 4; ++q) nl[q] = l[nw[q]];
                tet_idx[t] = make_uint2((unsigned)nl[0] | ((unsigned)nl[1] << 16), (unsigned)nl[2] | ((unsigned)nl[3] << 16));
                // edge rest lengths in the new local pairs
                auto edge_at = [&](int u, int v) {
                    for (int m = 0; m < owned_n[t]; ++m) {
                        const int kk = owned[2 * t + m];
                        const int a = edge_idx[kk] & 0xffff, c = edge_idx[kk] >> 16;
                        if ((a == u && c == v) || (a == v && c == u)) return kk;
                    }
                    return -1;
                };
                const int eAB = edge_at(nl[0], nl[1]);
                float4 ed = make_float4(edge_la[eAB].x, edge_la[eAB].y, 0.0f, 0.0f);
                if (cls == 2) {
                    const int eCD = edge_at(nl[2], nl[3]);
                    ed.z = edge_la[eCD].x; ed.w = edge_la[eCD].y;
                } else if (cls == 3) {
                    const int eAC = edge_at(nl[0], nl[2]);
                    ed.z = -edge_la[eAC].x; ed.w = edge_la[eAC].y;
                }
                tet_ed[t] = ed;
                tet_cls[t] = (unsigned char)cls;
                // Neo-Hookean tables for the new order: Ds' = Ds P with
                // P[k-1][m-1] = [nw[m] == k] - [nw[0] == k], so Dm'^-1 = P^-1 Dm^-1
                if (nh) {
                    const float* f = hm->tetrahedron_dm_inv + 9ll * t;
                    double d[9], P[9], Pi[9], d2[9];
                    for (int k = 0; k < 9; ++k) d[k] = f[k];
                    for (int k = 1; k <= 3; ++k)
                        for (int m = 1; m <= 3; ++m)
                            P[3 * (k - 1) + (m - 1)] = (nw[m] == k ? 1.0 : 0.0) - (nw[0] == k ? 1.0 : 0.0);
                    const double det = P[0] * (P[4] * P[8] - P[5] * P[7]) - P[1] * (P[3] * P[8] - P[5] * P[6]) +
                                       P[2] * (P[3] * P[7] - P[4] * P[6]);
                    Pi[0] = (P[4] * P[8] - P[5] * P[7]) / det; Pi[1] = (P[2] * P[7] - P[1] * P[8]) / det;
                    Pi[2] = (P[1] * P[5] - P[2] * P[4]) / det; Pi[3] = (P[5] * P[6] - P[3] * P[8]) / det;
                    Pi[4] = (P[0] * P[8] - P[2] * P[6]) / det; Pi[5] = (P[2] * P[3] - P[0] * P[5]) / det;
                    Pi[6] = (P[3] * P[7] - P[4] * P[6]) / det; Pi[7] = (P[1] * P[6] - P[0] * P[7]) / det;
                    Pi[8] = (P[0] * P[4] - P[1] * P[3]) / det;
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j)
                            d2[3 * i + j] = Pi[3 * i] * d[j] + Pi[3 * i + 1] * d[3 + j] + Pi[3 * i + 2] * d[6 + j];
                    auto mm = [&](int i, int j) {
                        return d2[3 * i] * d2[3 * j] + d2[3 * i + 1] * d2[3 * j + 1] + d2[3 * i + 2] * d2[3 * j + 2];
                    };
                    const double dd = d2[0] * (d2[4] * d2[8] - d2[5] * d2[7]) - d2[1] * (d2[3] * d2[8] - d2[5] * d2[6]) +
                                      d2[2] * (d2[3] * d2[7] - d2[4] * d2[6]);
                    nh0[t] = make_float4((float)mm(0, 0), (float)mm(0, 1), (float)mm(0, 2), (float)mm(1, 1));
                    nh1[t] = make_float4((float)mm(1, 2), (float)mm(2, 2), (float)dd, nh1[t].w);
                }
            }
            r.e0 = ne_new0;
            r.ne = (int)n_edge_idx.size() - ne_new0;
        }
        edge_idx.swap(n_edge_idx);
        edge_la.swap(n_edge_la);
    }

    // ---- order each env's constraint records by a greedy vertex colouring ----
    std::vector<int> tet_orig(T), edge_orig(edge_idx.size());
    {
        std::vector<uint64_t> used;
        std::vector<int> col;
        for (int e = 0; e < N; ++e) {
            const EnvRec& r = env[e];
            if (dup_of[e] >= 0) {
                const EnvRec& src = env[dup_of[e]];
                for (int j = 0; j < r.nt; ++j) tet_orig[r.t0 + j] = r.t0 + (tet_orig[src.t0 + j] - src.t0);
                for (int j = 0; j < r.ne; ++j) edge_orig[r.e0 + j] = r.e0 + (edge_orig[src.e0 + j] - src.e0);
                continue;
            }
            used.assign(r.nv, 0);
            col.resize(std::max(r.nt, r.ne));
            for (int t = 0; t < r.nt; ++t) {
                uint2 ix = tet_idx[r.t0 + t];
                int l[4] = {(int)(ix.x & 0xffff), (int)(ix.x >> 16), (int)(ix.y & 0xffff), (int)(ix.y >> 16)};
                uint64_t m = used[l[0]] | used[l[1]] | used[l[2]] | used[l[3]];
                int c = (~m) ? __builtin_ctzll(~m) : 63;
                col[t] = c;
                for (int k = 0; k < 4; ++k) used[l[k]] |= 1ull << c;
            }
            std::vector<int> ord(r.nt);
            std::iota(ord.begin(), ord.end(), 0);
            std::stable_sort(ord.begin(), ord.end(), [&](int a, int c2) {
                return col[a] != col[c2] ? col[a] < col[c2] : tet_cls[r.t0 + a] < tet_cls[r.t0 + c2];
            });
            bank_regroup(
                ord, 4,
                [&](int t, int c) {
                    const uint2 ix = tet_idx[r.t0 + t];
                    const unsigned w = c < 2 ? ix.x : ix.y;
                    return (int)((c & 1) ? (w >> 16) : (w & 0xffff));
                },
                [&](int t) { return col[t] * 4 + tet_cls[r.t0 + t]; });
            for (int j = 0; j < r.nt; ++j) tet_orig[r.t0 + j] = r.t0 + ord[j];
            used.assign(r.nv, 0);
            for (int k = 0; k < r.ne; ++k) {
                unsigned ix = edge_idx[r.e0 + k];
                int a = ix & 0xffff, c2 = ix >> 16;
                uint64_t m = used[a] | used[c2];
                int c = (~m) ? __builtin_ctzll(~m) : 63;
                col[k] = c;
                used[a] |= 1ull << c; used[c2] |= 1ull << c;
            }
            ord.resize(r.ne);
            std::iota(ord.begin(), ord.end(), 0);
            std::stable_sort(ord.begin(), ord.end(), [&](int a, int c2) { return col[a] < col[c2]; });
            bank_regroup(
                ord, 2,
                [&](int k, int c) {
                    const unsigned ix = edge_idx[r.e0 + k];
                    return (int)(c ? (ix >> 16) : (ix & 0xffff));
                },
                [&](int k) { return col[k]; });
            for (int j = 0; j < r.ne; ++j) edge_orig[r.e0 + j] = r.e0 + ord[j];
        }
        auto permute = [](auto& v, const std::vector<int>& orig) {
            if (v.empty()) return;
            auto c = v;
            for (size_t i = 0; i < orig.size(); ++i) v[i] = c[orig[i]];
        };
        permute(tet_idx, tet_orig); permute(tet_va, tet_orig); permute(nh0, tet_orig); permute(nh1, tet_orig);
        permute(tet_vs, tet_orig); permute(tet_ed, tet_orig); permute(edge_idx, edge_orig); permute(edge_la, edge_orig);
    }

    // ---- share identical constraint tables: envs of one mesh read the same records ----
    {
        for (int e = 0; e < N; ++e) {
            env[e].mt0 = env[e].t0;
            env[e].me0 = env[e].e0;
            for (int j = 0; j < env[e].nt; ++j) tet_orig[env[e].t0 + j] -= env[e].t0;
            for (int j = 0; j < env[e].ne; ++j) edge_orig[env[e].e0 + j] -= env[e].e0;
        }
        auto fnv = [](uint64_t h, const void* p, size_t n) {
            const unsigned char* c = static_cast<const unsigned char*>(p);
            for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
            return h;
        };
        auto same = [&](const EnvRec& a, const EnvRec& c) {
            auto eq = [](const auto& v, int o1, int o2, int n) {
                return n == 0 || v.empty() || std::memcmp(&v[o1], &v[o2], sizeof(v[0]) * (size_t)n) == 0;
            };
            return a.nv == c.nv && a.nt == c.nt && a.ne == c.ne && a.nf == c.nf &&
                   eq(tet_idx, a.t0, c.t0, a.nt) && eq(tet_va, a.t0, c.t0, a.nt) && eq(nh0, a.t0, c.t0, a.nt) &&
                   eq(nh1, a.t0, c.t0, a.nt) && eq(tet_vs, a.t0, c.t0, a.nt) && eq(tet_ed, a.t0, c.t0, a.nt) &&
                   eq(tet_orig, a.t0, c.t0, a.nt) && eq(edge_idx, a.e0, c.e0, a.ne) && eq(edge_la, a.e0, c.e0, a.ne) &&
                   eq(edge_orig, a.e0, c.e0, a.ne) && eq(tri_idx, a.f0, c.f0, a.nf);
        };
        std::vector<uint2> c_tet_idx; std::vector<float2> c_tet_va; std::vector<float4> c_nh0, c_nh1;
        std::vector<float> c_tet_vs; std::vector<float4> c_tet_ed; std::vector<int> c_tet_orig, c_edge_orig;
        std::vector<unsigned> c_edge_idx; std::vector<float2> c_edge_la; std::vector<uint2> c_tri_idx;
        std::unordered_map<uint64_t, std::vector<int>> seen;
        std::vector<EnvRec> out = env;
        auto app = [](auto& dst, const auto& src, int o, int n) {
            if (!src.empty()) dst.insert(dst.end(), src.begin() + o, src.begin() + o + n);
        };
        for (int e = 0; e < N; ++e) {
            const EnvRec& r = env[e];
            uint64_t h = fnv(1469598103934665603ull, &r.nv, sizeof(int) * 1);
            h = fnv(h, &r.nt, sizeof(int));
            h = fnv(h, &r.ne, sizeof(int));
            if (r.nt) h = fnv(h, &tet_idx[r.t0], sizeof(uint2) * (size_t)r.nt);
            int match = -1;
            for (int c : seen[h])
                if (same(r, env[c])) { match = c; break; }
            if (match >= 0) {
                out[e].t0 = out[match].t0; out[e].e0 = out[match].e0; out[e].f0 = out[match].f0;
                continue;
            }
            seen[h].push_back(e);
            out[e].t0 = (int)c_tet_idx.size(); out[e].e0 = (int)c_edge_idx.size(); out[e].f0 = (int)c_tri_idx.size();
            app(c_tet_idx, tet_idx, r.t0, r.nt); app(c_tet_va, tet_va, r.t0, r.nt); app(c_nh0, nh0, r.t0, r.nt);
            app(c_nh1, nh1, r.t0, r.nt); app(c_tet_vs, tet_vs, r.t0, r.nt); app(c_tet_ed, tet_ed, r.t0, r.nt);
            app(c_tet_orig, tet_orig, r.t0, r.nt); app(c_edge_idx, edge_idx, r.e0, r.ne);
            app(c_edge_la, edge_la, r.e0, r.ne); app(c_edge_orig, edge_orig, r.e0, r.ne);
            app(c_tri_idx, tri_idx, r.f0, r.nf);
        }
        env = out;
        tet_idx.swap(c_tet_idx); tet_va.swap(c_tet_va); nh0.swap(c_nh0); nh1.swap(c_nh1);
        tet_vs.swap(c_tet_vs); tet_ed.swap(c_tet_ed); tet_orig.swap(c_tet_orig); edge_idx.swap(c_edge_idx); edge_la.swap(c_edge_la);
        edge_orig.swap(c_edge_orig); tri_idx.swap(c_tri_idx);
    }

    // size classes: mode by fit, then by vertex-count band
    const int bands[] = {192, 384, 768, 1536, 3072, 65536};
    b->env_class.assign(N, -1);
    std::vector<std::vector<int>> members;
    std::vector<int> keys;  // mode*16 + band
    auto mode_for = [&](int nv) {
        if (precision == 64) return smem_bytes<double>(0, nv) <= dyn_budget ? 0 : 2;
        if (smem_bytes<float>(0, nv) <= dyn_budget) return 0;
        if (smem_bytes<float>(1, nv) <= dyn_budget) return 1;
        return 2;
    };
    for (int e = 0; e < N; ++e) {
        int m = mode_for(env[e].nv);
        int band = 0;
        while (env[e].nv > bands[band]) ++band;
        int key = m * 16 + (m == 0 ? band : 0);
        auto it = std::find(keys.begin(), keys.end(), key);
        int ci;
        if (it == keys.end()) { keys.push_back(key); members.emplace_back(); ci = (int)keys.size() - 1; }
        else ci = (int)(it - keys.begin());
        members[ci].push_back(e);
    }
    // order classes by key for reproducible launch order
    std::vector<int> order(keys.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int c) { return keys[a] < keys[c]; });
    size_t scratch_total = 0;
    b->env_cost.resize(N);
    for (int e = 0; e < N; ++e) b->env_cost[e] = 4ll * env[e].nt + env[e].ne + env[e].nf + env[e].nv;
    for (int oi : order) {
        auto& mem = members[oi];
        std::sort(mem.begin(), mem.end(), [&](int a, int c) {
            return b->env_cost[a] != b->env_cost[c] ? b->env_cost[a] > b->env_cost[c] : a < c;
        });
        ffsrl_batch::Class c{};
        c.mode = keys[oi] / 16;
        c.max_nv = 1;
        for (int e : mem) c.max_nv = std::max(c.max_nv, env[e].nv);
        c.smem = precision == 64 ? smem_bytes<double>(c.mode, c.max_nv) : smem_bytes<float>(c.mode, c.max_nv);
        if (p->flags & FFSRL_COLLIDE) {
            // the contact scan reads every surface triangle in every iteration: keep the
            // env's triangles in shared memory when they fit
            int max_nf = 0;
            for (int e : mem) max_nf = std::max(max_nf, env[e].nf);
            const size_t with = ((c.smem + 7) & ~(size_t)7) + 8 * (size_t)max_nf;
            if (max_nf > 0 && with <= dyn_budget) { c.tri_cap = max_nf; c.smem = with; }
        }
        c.scratch_stride = precision == 64 ? scratch_bytes<double>(c.mode, c.max_nv) : scratch_bytes<float>(c.mode, c.max_nv);
        c.scratch_stride = (c.scratch_stride + 255) & ~(size_t)255;
        c.members = (int)mem.size();
        int want = block_override > 0 ? block_override : default_block(c.max_nv, c.mode);
        if (int32_t st = configure_class(b, c, want, dyn_budget)) { free_batch(b); return st; }
        // scratch for the largest grid any block size can give (8 resident blocks per SM)
        c.scratch_offset = scratch_total;
        if (c.scratch_stride) scratch_total += c.scratch_stride * (size_t)std::min(c.members, 8 * b->sm_count);
        c.work_offset = (int)b->work_host.size();
        c.work_count = (int)mem.size();
        for (int e : mem) { b->env_class[e] = (int)b->classes.size(); b->work_host.push_back(e); }
        b->classes.push_back(c);
    }

    int32_t st = FFSRL_OK;
    if ((st = dalloc(b, &b->d_cnt0, (size_t)V)) || (st = upload(b->d_cnt0, cnt0)) ||
        (st = dalloc(b, &b->d_tet_orig, tet_orig.size())) || (st = upload(b->d_tet_orig, tet_orig)) ||
        (st = dalloc(b, &b->d_edge_orig, edge_orig.size())) || (st = upload(b->d_edge_orig, edge_orig)) ||
        (st = dalloc(b, &b->d_env, N)) || (st = upload(b->d_env, env)) ||
        (st = dalloc(b, &b->d_tet_idx, tet_idx.size())) || (st = upload(b->d_tet_idx, tet_idx)) ||
        (st = dalloc(b, &b->d_tet_va, tet_va.size())) || (st = upload(b->d_tet_va, tet_va)) ||
        (st = dalloc(b, &b->d_nh0, nh0.size())) || (st = upload(b->d_nh0, nh0)) ||
        (st = dalloc(b, &b->d_nh1, nh1.size())) || (st = upload(b->d_nh1, nh1)) ||
        (st = dalloc(b, &b->d_tet_vs, tet_vs.size())) || (st = upload(b->d_tet_vs, tet_vs)) ||
        (st = dalloc(b, &b->d_tet_ed, tet_ed.size())) || (st = upload(b->d_tet_ed, tet_ed)) ||
        (st = dalloc(b, &b->d_edge_idx, edge_idx.size())) || (st = upload(b->d_edge_idx, edge_idx)) ||
        (st = dalloc(b, &b->d_edge_la, edge_la.size())) || (st = upload(b->d_edge_la, edge_la)) ||
        (st = dalloc(b, &b->d_tri_idx, tri_idx.size())) || (st = upload(b->d_tri_idx, tri_idx)) ||
        (st = dalloc(b, &b->d_conn_idx, conn_idx.size())) || (st = upload(b->d_conn_idx, conn_idx)) ||
        (st = dalloc(b, &b->d_conn_bar, conn_bar.size())) || (st = upload(b->d_conn_bar, conn_bar)) ||
        (st = dalloc(b, &b->d_conn_vert, conn_vert.size())) || (st = upload(b->d_conn_vert, conn_vert)) ||
        (st = dalloc(b, &b->d_pend, conn ? 3 * (size_t)V : 0)) || (st = dalloc(b, &b->d_pcnt, conn ? (size_t)V : 0)) ||
        (st = dalloc(b, &b->d_work, (size_t)N)) || (st = upload(b->d_work, b->work_host)) ||
        (st = dalloc(b, &b->d_status, (size_t)N)) ||
        (st = dalloc(b, &b->d_scratch, scratch_total * kLanes))) {
        free_batch(b);
        return st;
    }
    FFSRL_CUDA_TRY(cudaMemset(b->d_status, 0, sizeof(int) * N));
    if (conn) {
        FFSRL_CUDA_TRY(cudaMemset(b->d_pend, 0, sizeof(int) * 3 * (size_t)V));
        FFSRL_CUDA_TRY(cudaMemset(b->d_pcnt, 0, sizeof(int) * (size_t)V));
    }
    if (precision == 64) {
        if ((st = dalloc(b, &b->d_state64, 9 * (size_t)V))) { free_batch(b); return st; }
        // double state initialised from the model's float state
        std::vector<float> hx(3 * V), hv(3 * V);
        std::vector<double> h64(9 * V);
        cudaMemcpy(hx.data(), dmod->vertex, 12 * V, cudaMemcpyDeviceToHost);
        cudaMemcpy(hv.data(), dmod->velocity, 12 * V, cudaMemcpyDeviceToHost);
        for (int64_t i = 0; i < 3 * V; ++i) { h64[i] = hx[i]; h64[3 * V + i] = hv[i]; h64[6 * V + i] = hx[i]; }
        if ((st = upload(b->d_state64, h64))) { free_batch(b); return st; }
    }
    b->scratch_per_lane = scratch_total;
    b->lanes.resize(kLanes);
    for (auto& L : b->lanes) {
        if ((st = dalloc(b, &L.d_counters, b->classes.size() + 1)) || (st = dalloc(b, &L.d_work_sub, (size_t)N))) {
            free_batch(b);
            return st;
        }
        FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_work_pinned, sizeof(int) * N, cudaHostAllocDefault));
        FFSRL_CUDA_TRY(cudaEventCreateWithFlags(&L.fork, cudaEventDisableTiming));
        FFSRL_CUDA_TRY(cudaEventCreateWithFlags(&L.staged, cudaEventDisableTiming));
        L.streams.resize(b->classes.size());
        L.done.resize(b->classes.size());
        for (size_t ci = 0; ci < b->classes.size(); ++ci) {
            FFSRL_CUDA_TRY(cudaStreamCreateWithFlags(&L.streams[ci], cudaStreamNonBlocking));
            FFSRL_CUDA_TRY(cudaEventCreateWithFlags(&L.done[ci], cudaEventDisableTiming));
        }
    }
    *out = b;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_destroy(ffsrl_batch* b) {
    if (b) cudaDeviceSynchronize();
    free_batch(b);
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_step(ffsrl_batch* b, int32_t n_steps, void* stream) {
    if (!b || n_steps < 0) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_step");
    if (n_steps == 0) return FFSRL_OK;
    std::vector<int> counts, offsets;
    for (auto& c : b->classes) { counts.push_back(c.work_count); offsets.push_back(c.work_offset); }
    return run(b, 0, counts, b->d_work, offsets, n_steps, (cudaStream_t)stream);
}

extern "C" int32_t ffsrl_batch_step_envs_lane(ffsrl_batch* b, int32_t lane, const int32_t* env_ids, int32_t n,
                                              int32_t n_steps, void* stream) {
    if (!b || n < 0 || n_steps < 0 || (n > 0 && !env_ids) || lane < 0 || lane >= (int)b->lanes.size())
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_step_envs: bad argument or lane");
    if (n == 0 || n_steps == 0) return FFSRL_OK;
    if (n > b->num_envs) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_step_envs: more ids than envs");
    cudaStream_t s = (cudaStream_t)stream;
    auto& L = b->lanes[lane];
    std::vector<std::vector<int>> per(b->classes.size());
    for (int i = 0; i < n; ++i) {
        int e = env_ids[i];
        if (e < 0 || e >= b->num_envs) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_step_envs: env id out of range");
        per[b->env_class[e]].push_back(e);
    }
    // the lane's pinned staging buffer is reused: wait until its previous upload has read it
    if (L.staged_pending) FFSRL_CUDA_TRY(cudaEventSynchronize(L.staged));
    std::vector<int> counts, offsets;
    int o = 0;
    for (size_t ci = 0; ci < per.size(); ++ci) {
        auto& v = per[ci];
        std::sort(v.begin(), v.end(), [&](int a, int c) {
            return b->env_cost[a] != b->env_cost[c] ? b->env_cost[a] > b->env_cost[c] : a < c;
        });
        offsets.push_back(o);
        counts.push_back((int)v.size());
        for (int e : v) L.h_work_pinned[o++] = e;
    }
    FFSRL_CUDA_TRY(cudaMemcpyAsync(L.d_work_sub, L.h_work_pinned, sizeof(int) * o, cudaMemcpyHostToDevice, s));
    FFSRL_CUDA_TRY(cudaEventRecord(L.staged, s));
    L.staged_pending = true;
    return run(b, lane, counts, L.d_work_sub, offsets, n_steps, s);
}

extern "C" int32_t ffsrl_batch_step_envs(ffsrl_batch* b, const int32_t* env_ids, int32_t n, int32_t n_steps,
                                         void* stream) {
    return ffsrl_batch_step_envs_lane(b, 0, env_ids, n, n_steps, stream);
}

extern "C" int32_t ffsrl_batch_info(const ffsrl_batch* b, int64_t* device_bytes, int32_t* num_classes,
                                    int32_t* block_threads) {
    if (!b) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_info");
    if (device_bytes) *device_bytes = b->device_bytes;
    if (num_classes) *num_classes = (int32_t)b->classes.size();
    if (block_threads)
        for (size_t i = 0; i < b->classes.size(); ++i) block_threads[i] = b->classes[i].block;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_env_status(const ffsrl_batch* b, int32_t* host_status, int32_t num_envs) {
    if (!b || !host_status || num_envs != b->num_envs) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_env_status");
    FFSRL_CUDA_TRY(cudaMemcpy(host_status, b->d_status, sizeof(int) * num_envs, cudaMemcpyDeviceToHost));
    return FFSRL_OK;
}

// Copies the float64 plan's state (x, v, predicted; each [3V]) to host memory.
extern "C" int32_t ffsrl_batch_state_f64(const ffsrl_batch* b, double* host_xvx) {
    if (!b || !host_xvx || b->precision != 64) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_state_f64: not a float64 plan");
    FFSRL_CUDA_TRY(cudaMemcpy(host_xvx, b->d_state64, sizeof(double) * 9 * (size_t)b->dm.num_vertices, cudaMemcpyDeviceToHost));
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_class_info(const ffsrl_batch* b, int32_t cls, int32_t* max_nv, int32_t* mode,
                                          int32_t* block, int32_t* num_envs) {
    if (!b || cls < 0 || cls >= (int)b->classes.size()) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_class_info");
    const auto& c = b->classes[cls];
    if (max_nv) *max_nv = c.max_nv;
    if (mode) *mode = c.mode;
    if (block) *block = c.block;
    if (num_envs) *num_envs = c.work_count;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_class_envs(const ffsrl_batch* b, int32_t cls, int32_t* env_ids) {
    if (!b || !env_ids || cls < 0 || cls >= (int)b->classes.size())
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_class_envs");
    const auto& c = b->classes[cls];
    for (int i = 0; i < c.work_count; ++i) env_ids[i] = b->work_host[c.work_offset + i];
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_set_class_prefetch(ffsrl_batch* b, int32_t cls, int32_t kind) {
    if (!b || cls < 0 || cls >= (int)b->classes.size() || kind < 0 || kind > 2)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_set_class_prefetch");
    if (kind == 2 && b->precision == 64)
        return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch_set_class_prefetch: no float64 register pipeline");
    FFSRL_CUDA_TRY(cudaDeviceSynchronize());
    ffsrl_batch::Class c = b->classes[cls];
    c.prefetch = kind;
    if (int32_t st = configure_class(b, c, c.block, b->dyn_budget)) return st;
    b->classes[cls] = c;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_batch_set_class_block(ffsrl_batch* b, int32_t cls, int32_t block) {
    if (!b || cls < 0 || cls >= (int)b->classes.size()) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_set_class_block");
    FFSRL_CUDA_TRY(cudaDeviceSynchronize());
    ffsrl_batch::Class c = b->classes[cls];
    if (int32_t st = configure_class(b, c, block, b->dyn_budget)) return st;
    b->classes[cls] = c;
    return FFSRL_OK;
}
