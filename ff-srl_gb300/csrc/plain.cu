// plain.cu -- reference-shaped step: one kernel launch per reference kernel, in the
// launch order of SimIntegratorDO.stepModel (FF_SRL/FF_SRL/integrator.py:1640-1741),
// per-vertex corrections accumulated with float atomics as the reference does.  This is
// the drop-in that the batched form (batched.cu) is measured against.
#include <cuda_runtime.h>
#include <cstdint>
#include <mutex>
#include <string>
#include "ffsrl_internal.h"
#include "vecmath.cuh"

namespace ffsrl {
namespace {

constexpr int kBlock = 256;

// gravity (integrator.py:40-63)
__global__ void k_gravity(const float* __restrict__ x, float* __restrict__ xp, const float* __restrict__ vel,
                          const float* __restrict__ inv_mass, v3 g, float damping, float dt, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 p = ld3(x, i), v = ld3(vel, i);
    float inv = inv_mass[i];
    float damp = 1.0f - damping;
    v = v + g * inv * dt * damp;
    if (inv < FFSRL_FLOAT_EPS) v = mk(0.0f, 0.0f, 0.0f);
    st3(xp, i, p + v * dt);
}

// volumeConstraints (integrator.py:444-504)
__global__ void k_volume(const float* __restrict__ xp, float* dp, int* cnt, const int* __restrict__ tet,
                         const float* __restrict__ rest, const float* __restrict__ inv_mass,
                         const float* __restrict__ active_tet, float ks, int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float active = active_tet[t];
    if (!(active == 1.0f)) return;
    int4 id = reinterpret_cast<const int4*>(tet)[t];
    v3 pa = ld3(xp, id.x), pb = ld3(xp, id.y), pc = ld3(xp, id.z), pd = ld3(xp, id.w);
    float rv = rest[t];
    v3 p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
    v3 q2 = cross(p3, p1), q1 = cross(p2, p3), q3 = cross(p1, p2);
    v3 q0 = -q1 - q2 - q3;
    float mA = inv_mass[id.x], mB = inv_mass[id.y], mC = inv_mass[id.z], mD = inv_mass[id.w];
    float vol = fabsf(dot(cross(p1, p2), p3)) / 6.0f;
    float w = mA * dot(q0, q0) + mB * dot(q1, q1) + mC * dot(q2, q2) + mD * dot(q3, q3);
    if (fabsf(w) < FFSRL_FLOAT_EPS) return;
    float C = rv - vol;
    float dl = -ks * active * C / w;
    atomic_add3_pair(dp, id.x, q0 * dl * mA);
    atomic_add3_pair(dp, id.y, q1 * dl * mB);
    atomic_add3_pair(dp, id.z, q2 * dl * mC);
    atomic_add3_pair(dp, id.w, q3 * dl * mD);
    atomicAdd(cnt + id.x, 1); atomicAdd(cnt + id.y, 1); atomicAdd(cnt + id.z, 1); atomicAdd(cnt + id.w, 1);
}

// volumeConstraintsXPBD (integrator.py:507-576), signed rest volume
__global__ void k_volume_xpbd(const float* __restrict__ xp, float* dp, int* cnt, float* lam,
                              const int* __restrict__ tet, const float* __restrict__ rest,
                              const float* __restrict__ inv_mass, const float* __restrict__ active_tet, float alpha,
                              int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (!(active_tet[t] == 1.0f)) return;
    int4 id = reinterpret_cast<const int4*>(tet)[t];
    v3 pa = ld3(xp, id.x), pb = ld3(xp, id.y), pc = ld3(xp, id.z), pd = ld3(xp, id.w);
    float rv = rest[t];
    float l0 = lam[t];
    v3 p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
    v3 q2 = cross(p3, p1), q1 = cross(p2, p3), q3 = cross(p1, p2);
    v3 q0 = -q1 - q2 - q3;
    float mA = inv_mass[id.x], mB = inv_mass[id.y], mC = inv_mass[id.z], mD = inv_mass[id.w];
    float vol = dot(cross(p1, p2), p3) / 6.0f;
    float w = mA * dot(q0, q0) + mB * dot(q1, q1) + mC * dot(q2, q2) + mD * dot(q3, q3);
    if (fabsf(w) < FFSRL_FLOAT_EPS) return;
    float C = vol - rv;
    float dl = -(C + alpha * l0) / (w + alpha);
    lam[t] = l0 + dl;
    atomic_add3_pair(dp, id.x, q0 * dl * mA);
    atomic_add3_pair(dp, id.y, q1 * dl * mB);
    atomic_add3_pair(dp, id.z, q2 * dl * mC);
    atomic_add3_pair(dp, id.w, q3 * dl * mD);
    atomicAdd(cnt + id.x, 1); atomicAdd(cnt + id.y, 1); atomicAdd(cnt + id.z, 1); atomicAdd(cnt + id.w, 1);
}

// neoHookeanConstraints (integrator.py:578-698): stable Neo-Hookean hydrostatic +
// deviatoric pair with F = [p1 p2 p3] Dm^-1; lambda starts at 0 every projection
// because the reference never stores it.
__global__ void k_neohookean(const float* __restrict__ xp, float* dp, int* cnt, const int* __restrict__ tet,
                             const float* __restrict__ rest, const float* __restrict__ inv_mass,
                             const float* __restrict__ dm_inv, float vol_c, float dev_c, float dt, int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int4 id = reinterpret_cast<const int4*>(tet)[t];
    float rv = rest[t];
    v3 pa = ld3(xp, id.x), pb = ld3(xp, id.y), pc = ld3(xp, id.z), pd = ld3(xp, id.w);
    v3 p1 = pb - pa, p2 = pc - pa, p3 = pd - pa;
    float mA = inv_mass[id.x], mB = inv_mass[id.y], mC = inv_mass[id.z], mD = inv_mass[id.w];
    const float* D = dm_inv + 9ll * t;
    float d00 = D[0], d01 = D[1], d02 = D[2], d10 = D[3], d11 = D[4], d12 = D[5], d20 = D[6], d21 = D[7], d22 = D[8];
    v3 f0 = p1 * d00 + p2 * d10 + p3 * d20;
    v3 f1 = p1 * d01 + p2 * d11 + p3 * d21;
    v3 f2 = p1 * d02 + p2 * d12 + p3 * d22;
    v3 c0 = cross(f1, f2), c1 = cross(f2, f0), c2 = cross(f0, f1);
    v3 g1 = c0 * d00 + c1 * d01 + c2 * d02;
    v3 g2 = c0 * d10 + c1 * d11 + c2 * d12;
    v3 g3 = c0 * d20 + c1 * d21 + c2 * d22;
    v3 g0 = -g1 - g2 - g3;
    float detF = dot(f0, c0);
    float invVol = 1.0f / vol_c, invDev = 1.0f / dev_c;
    float C = detF - 1.0f - invDev / invVol;
    float w = 0.0f, l;
    l = length(g0); w += l * l * mA;
    l = length(g1); w += l * l * mB;
    l = length(g2); w += l * l * mC;
    l = length(g3); w += l * l * mD;
    if (w < FFSRL_FLOAT_EPS) return;
    float alpha = vol_c / dt / dt / rv;
    float dl = -C / (w + alpha);
    v3 dA = g0 * dl * mA, dB = g1 * dl * mB, dC = g2 * dl * mC, dD = g3 * dl * mD;
    float l0 = length(f0), l1 = length(f1), l2 = length(f2);
    float rs = sqrtf(l0 * l0 + l1 * l1 + l2 * l2);
    float rsi = 1.0f / rs;
    C = rs;
    g1 = (f0 * d00 + f1 * d01 + f2 * d02) * rsi;
    g2 = (f0 * d10 + f1 * d11 + f2 * d12) * rsi;
    g3 = (f0 * d20 + f1 * d21 + f2 * d22) * rsi;
    g0 = -g1 - g2 - g3;
    w = 0.0f;
    l = length(g0); w += l * l * mA;
    l = length(g1); w += l * l * mB;
    l = length(g2); w += l * l * mC;
    l = length(g3); w += l * l * mD;
    if (w < FFSRL_FLOAT_EPS) return;
    alpha = dev_c / dt / dt / rv;
    dl = -C / (w + alpha);
    dA = dA + g0 * dl * mA; dB = dB + g1 * dl * mB; dC = dC + g2 * dl * mC; dD = dD + g3 * dl * mD;
    atomic_add3_pair(dp, id.x, dA); atomic_add3_pair(dp, id.y, dB); atomic_add3_pair(dp, id.z, dC); atomic_add3_pair(dp, id.w, dD);
    atomicAdd(cnt + id.x, 1); atomicAdd(cnt + id.y, 1); atomicAdd(cnt + id.z, 1); atomicAdd(cnt + id.w, 1);
}

// distanceConstraints (integrator.py:65-109)
__global__ void k_distance(const float* __restrict__ xp, float* dp, int* cnt, const int* __restrict__ edge,
                           const float* __restrict__ rest, const float* __restrict__ inv_mass,
                           const float* __restrict__ active_edge, float ks, int n) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    float active = active_edge[e];
    if (active == 0.0f) return;
    int2 id = reinterpret_cast<const int2*>(edge)[e];
    v3 pa = ld3(xp, id.x), pb = ld3(xp, id.y);
    float L0 = rest[e];
    if (L0 < FFSRL_FLOAT_EPS) return;
    v3 dir = pb - pa;
    float len = length(dir);
    if (len < FFSRL_FLOAT_EPS) return;
    float mA = inv_mass[id.x], mB = inv_mass[id.y];
    float w = mA + mB;
    if (w < FFSRL_FLOAT_EPS) return;
    float C = len - L0;
    v3 d = -C * (dir / len) * ks * active / w;
    atomic_add3_pair(dp, id.x, -(d * mA));
    atomic_add3_pair(dp, id.y, d * mB);
    atomicAdd(cnt + id.x, 1); atomicAdd(cnt + id.y, 1);
}

// distanceConstraintsXPBD (integrator.py:191-240)
__global__ void k_distance_xpbd(const float* __restrict__ xp, float* dp, int* cnt, float* lam,
                                const int* __restrict__ edge, const float* __restrict__ rest,
                                const float* __restrict__ inv_mass, const float* __restrict__ active_edge,
                                float alpha, int n) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    if (active_edge[e] == 0.0f) return;
    int2 id = reinterpret_cast<const int2*>(edge)[e];
    v3 pa = ld3(xp, id.x), pb = ld3(xp, id.y);
    float L0 = rest[e];
    if (L0 < FFSRL_FLOAT_EPS) return;
    float l0 = lam[e];
    v3 dir = pb - pa;
    float len = length(dir);
    if (len < FFSRL_FLOAT_EPS) return;
    float mA = inv_mass[id.x], mB = inv_mass[id.y];
    float w = mA + mB;
    if (w < FFSRL_FLOAT_EPS) return;
    float C = len - L0;
    float dl = -(C + alpha * l0) / (w + alpha);
    lam[e] = l0 + dl;
    v3 d = dl * normalize(dir);
    atomic_add3_pair(dp, id.x, -(d * mA));
    atomic_add3_pair(dp, id.y, d * mB);
    atomicAdd(cnt + id.x, 1); atomicAdd(cnt + id.y, 1);
}

// applyConstraints (integrator.py:946-960)
__global__ void k_apply(float* __restrict__ xp, float* __restrict__ dp, int* __restrict__ cnt, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cnt[i];
    if (c > 0) {
        float N = float(c);
        v3 d = ld3(dp, i);
        st3(xp, i, ld3(xp, i) + mk(d.x / N, d.y / N, d.z / N));
    }
    st3(dp, i, mk(0.0f, 0.0f, 0.0f));
    cnt[i] = 0;
}

// dragConstraintsDO (integrator.py:412-442): pull toward laparoscopeTip[env*4 + 2]
__global__ void k_drag(float* __restrict__ xp, const float* __restrict__ drag, const int* __restrict__ v2e,
                       const float* __restrict__ tip, float ks, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float dr = drag[i];
    int env = v2e[i];
    if (dr == 0.0f) return;
    v3 pos = ld3(xp, i);
    v3 t = ld3(tip, 4ll * env + 2);
    v3 dir = pos - t;
    float len = length(dir);
    if (len < FFSRL_FLOAT_EPS) return;
    v3 d = len * normalize(dir) * dr * ks / 2.0f;
    st3(xp, i, pos - d);
}

// triToPointDistanceConstraintsDO (integrator.py:300-353)
__global__ void k_connector(const float* __restrict__ xp, float* dp, int* cnt, const int* __restrict__ tri_ids,
                            const float* __restrict__ bar, const int* __restrict__ pt_ids,
                            const float* __restrict__ rest, float wratio, float ks, float rmul, int n) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    int ta = tri_ids[3 * c], tb = tri_ids[3 * c + 1], tc = tri_ids[3 * c + 2];
    v3 A = ld3(xp, ta), B = ld3(xp, tb), Cc = ld3(xp, tc);
    v3 b = ld3(bar, c);
    v3 centre = A * b.x + B * b.y + Cc * b.z;
    int pid = pt_ids[c];
    v3 pos = ld3(xp, pid);
    float rd = rest[c];
    v3 dir = pos - centre;
    float len = length(dir);
    if (len < FFSRL_FLOAT_EPS) return;
    float wt = 1.0f - wratio;
    float C = len - rd * rmul;
    float s = wratio + wt * (b.x * b.x + b.y * b.y + b.z * b.z);
    v3 delta = (C / s) * (dir / len) * ks;
    atomic_add3_pair(dp, pid, -(delta * wratio));
    atomic_add3_pair(dp, ta, delta * wt * b.x);
    atomic_add3_pair(dp, tb, delta * wt * b.y);
    atomic_add3_pair(dp, tc, delta * wt * b.z);
    atomicAdd(cnt + pid, 1); atomicAdd(cnt + ta, 1); atomicAdd(cnt + tb, 1); atomicAdd(cnt + tc, 1);
}

// collideLaparoscopeDO (integrator.py:981-1050).  Responses go to a separate
// accumulator instead of straight into predictedVertex, so every triangle reads the
// positions as they were when the launch began; k_collide_apply subtracts them.
__global__ void k_collide(const float* __restrict__ xp, float* cdp, const int* __restrict__ tri,
                          const int* __restrict__ t2e, const int* __restrict__ hole,
                          const float* __restrict__ inv_mass, const float* __restrict__ base,
                          const float* __restrict__ tip, const float* __restrict__ radius, int* in_collision,
                          float ks, int n) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    int env = t2e[f];
    if (hole[f] == 1) return;
    int a = tri[3 * f], b = tri[3 * f + 1], c = tri[3 * f + 2];
    v3 pA = ld3(xp, a), pB = ld3(xp, b), pC = ld3(xp, c);
    v3 centre = (pA + pB + pC) * 0.3333f;
    v3 nrm = normalize(cross(pB - pA, pC - pA));
    v3 tA = mk(0.0f, 0.0f, 0.0f), tB = tA, tC = tA;
    float tl = 0.0f;
    for (int i = 0; i < 3; ++i) {
        long long k = 4ll * env + i;
        v3 rA = mk(0.0f, 0.0f, 0.0f), rB = rA, rC = rA;
        capsule_response(ld3(tip, k), ld3(base, k), radius[k], nrm, centre, pA, pB, pC, ks, rA, rB, rC);
        tA = tA + rA; tB = tB + rB; tC = tC + rC;
        tl = tl + length(rA) + length(rB) + length(rC);
    }
    if (tl > 0.0f) atomicAdd(in_collision + env, 1);
    if (inv_mass[a] > 0.0f) atomic_add3_pair(cdp, a, tA);
    if (inv_mass[b] > 0.0f) atomic_add3_pair(cdp, b, tB);
    if (inv_mass[c] > 0.0f) atomic_add3_pair(cdp, c, tC);
}

__global__ void k_collide_apply(float* __restrict__ xp, float* __restrict__ cdp, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    st3(xp, i, ld3(xp, i) - ld3(cdp, i));
    st3(cdp, i, mk(0.0f, 0.0f, 0.0f));
}

// bounds (integrator.py:12-21)
__global__ void k_bounds(float* __restrict__ xp, float ground, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (xp[3 * i + 1] < ground) xp[3 * i + 1] = ground;
}

// PBDStep (integrator.py:23-38)
__global__ void k_pbd(float* __restrict__ x, const float* __restrict__ xp, float* __restrict__ vel, float dt, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 p = ld3(x, i), q = ld3(xp, i);
    v3 v = (q - p) * (1.0f / dt);
    st3(x, i, q);
    st3(vel, i, v);
}

__global__ void k_zero(float* p, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) p[i] = 0.0f;
}

// remapAToBKernel (utils.py:32-42)
__global__ void k_remap(float* __restrict__ dst, const float* __restrict__ src, const int* __restrict__ map, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int a = map[2 * i], b = map[2 * i + 1];
    st3(dst, a, ld3(src, b));
}

// remapAToBKernel over one listed env's points per block
__global__ void k_remap_envs(float* __restrict__ dst, const float* __restrict__ src, const int* __restrict__ map,
                             const int* __restrict__ pstart, const int* __restrict__ ids, int num_envs) {
    int e = ids[blockIdx.x];
    if (e < 0 || e >= num_envs) return;
    for (int i = pstart[e] + threadIdx.x; i < pstart[e + 1]; i += blockDim.x) {
        int a = map[2 * i], b = map[2 * i + 1];
        st3(dst, a, ld3(src, b));
    }
}

// updateClampsDragKernel (modelDO.py:247-279)
__global__ void k_update_clamps(const float* __restrict__ pos, const int* __restrict__ v2e,
                                const float* __restrict__ tip, float* drag, float radius,
                                const int* __restrict__ state, const int* __restrict__ update, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int env = v2e[i];
    int id = env * 3;
    if (update[id] == 0) return;
    if (state[id] == 1) {
        float l = length(ld3(pos, i) - ld3(tip, 4ll * env + 3));
        drag[i] = l < radius ? 1.0f : 0.0f;
    } else {
        drag[i] = 0.0f;
    }
}

// forceClampsDragKernel (modelDO.py:281-289)
__global__ void k_force_clamps(float* drag, int vid, const int* __restrict__ env_id, float on, int vpe, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    drag[(long long)env_id[i] * vpe + vid] = on;
}

// One block per env: nearest candidate within radius of the drag point, ties to the
// lower candidate position.
__global__ void k_grasp_nearest(const float* __restrict__ pos, const int* __restrict__ cstart,
                                const int* __restrict__ cand, const float* __restrict__ tip,
                                const int* __restrict__ clamp, float radius, float* drag,
                                const int* __restrict__ ids, int num_envs) {
    const int k = blockIdx.x;        // clamp flag index
    const int e = ids ? ids[k] : k;  // env
    if (e < 0 || e >= num_envs) return;
    int c0 = cstart[e], c1 = cstart[e + 1];
    if (clamp[k] == 0) {
        for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) drag[cand[k]] = 0.0f;
        return;
    }
    v3 t = ld3(tip, 4ll * e + 3);
    unsigned long long best = ~0ull;
    for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
        float d = length(ld3(pos, cand[k]) - t);
        if (d < radius) {
            unsigned long long key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)(k - c0);
            best = key < best ? key : best;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other < best ? other : best;
    }
    __shared__ unsigned long long s_best[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_best[wid] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long b = ~0ull;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) b = s_best[w] < b ? s_best[w] : b;
        s_best[0] = b;
    }
    __syncthreads();
    unsigned long long b = s_best[0];
    for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x)
        drag[cand[k]] = (b != ~0ull && (unsigned)(k - c0) == (unsigned)(b & 0xffffffffu)) ? 1.0f : 0.0f;
}

// env-list variant: disp[i] moves env env_ids[i]
__global__ void k_move_tool_envs(float* base, float* tip, const float* __restrict__ disp, const int* __restrict__ ids,
                                 int n, int num_envs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * n) return;
    int k = i >> 2;
    if (ids[k] < 0 || ids[k] >= num_envs) return;
    long long slot = 4ll * ids[k] + (i & 3);
    v3 d = ld3(disp, k);
    st3(base, slot, ld3(base, slot) + d);
    st3(tip, slot, ld3(tip, slot) + d);
}

// one block per listed env: rest positions, zero velocity and grasp, initial instrument
__global__ void k_reset_envs(float* vertex, float* velocity, float* drag, const float* __restrict__ init,
                             float* base, float* tip, const float* __restrict__ init_base,
                             const float* __restrict__ init_tip, int* in_collision, float* xform,
                             const float* __restrict__ init_xform, const int* __restrict__ vstart,
                             const int* __restrict__ ids, int num_envs) {
    const int e = ids[blockIdx.x];
    if (e < 0 || e >= num_envs) return;
    const long long v0 = vstart[e], v1 = vstart[e + 1];
    for (long long i = 3 * v0 + threadIdx.x; i < 3 * v1; i += blockDim.x) {
        vertex[i] = init[i];
        velocity[i] = 0.0f;
    }
    for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x) drag[v] = 0.0f;
    if (threadIdx.x < 12) {
        const long long k = 12ll * e + threadIdx.x;
        base[k] = init_base[k];
        tip[k] = init_tip[k];
    }
    if (threadIdx.x == 0) in_collision[e] = 0;
    if (xform && threadIdx.x < 112) xform[112ll * e + threadIdx.x] = init_xform[112ll * e + threadIdx.x];
}

__global__ void k_move_tool(float* base, float* tip, const float* __restrict__ disp, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;  // one thread per (env, entry)
    if (i >= 4 * n) return;
    int e = i >> 2;
    v3 d = ld3(disp, e);
    st3(base, i, ld3(base, i) + d);
    st3(tip, i, ld3(tip, i) + d);
}

}  // namespace
}  // namespace ffsrl

using namespace ffsrl;

extern "C" int32_t ffsrl_step_model(const ffsrl_model* m, const ffsrl_params* p, void* stream_) {
    if (!m || !p) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: null model or params");
    if (p->substeps < 0 || p->iterations < 0) return fail(FFSRL_ERR_INVALID_ARGUMENT, "negative substeps/iterations");
    cudaStream_t s = (cudaStream_t)stream_;
    const int V = m->num_vertices, T = m->num_tetrahedrons, E = m->num_edges, F = m->num_triangles;
    const int C = m->num_connectors;
    const uint32_t fl = p->flags;
    if (V <= 0) return FFSRL_OK;
    if (!m->vertex || !m->predicted_vertex || !m->velocity || !m->dp || !m->constraints_number || !m->inverse_mass)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: missing state arrays");
    if ((fl & (FFSRL_VOLUME | FFSRL_NEOHOOKEAN | FFSRL_VOLUME_XPBD)) && T > 0 &&
        (!m->tetrahedron || !m->tetrahedron_rest_volume))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: missing tet arrays");
    if ((fl & (FFSRL_VOLUME | FFSRL_VOLUME_XPBD)) && T > 0 && !m->active_tetrahedron)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: missing active_tetrahedron");
    if ((fl & FFSRL_NEOHOOKEAN) && T > 0 && !m->tetrahedron_dm_inv)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: Neo-Hookean needs tetrahedron_dm_inv");
    if ((fl & FFSRL_VOLUME_XPBD) && T > 0 && (!m->tetrahedron_lambda || !m->xpbd_rest_volume))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: XPBD volume needs lambdas and signed rest volume");
    if ((fl & (FFSRL_DISTANCE | FFSRL_DISTANCE_XPBD)) && E > 0 && (!m->edge || !m->edge_rest_length || !m->active_edge))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: missing edge arrays");
    if ((fl & FFSRL_DISTANCE_XPBD) && E > 0 && !m->edge_lambda)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: XPBD distance needs edge_lambda");
    if ((fl & FFSRL_DRAG) && (!m->active_drag_constraint || !m->vertex_to_env || !m->laparoscope_tip))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: drag needs drag mask, vertex_to_env, tips");
    if ((fl & FFSRL_COLLIDE) && F > 0 &&
        (!m->triangle || !m->tri_to_env || !m->hole || !m->laparoscope_base || !m->laparoscope_tip ||
         !m->laparoscope_radius || !m->laparoscope_in_collision || !m->collision_dp))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: collision needs triangles, instrument, collision_dp");
    if ((fl & FFSRL_CONNECTORS) && C > 0 &&
        (!m->connector_triangle_id || !m->connector_tri_bar || !m->connector_vertex_id || !m->connector_rest_dist))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model: missing connector arrays");

    const v3 g = {p->gravity[0], p->gravity[1], p->gravity[2]};
    const float adist = (float)((double)p->distance_compliance / ((double)p->dt * (double)p->dt));
    const float avol = (float)((double)p->volume_compliance_xpbd / ((double)p->dt * (double)p->dt));
    const unsigned gv = grid_for(V, kBlock), gt = grid_for(T, kBlock), ge = grid_for(E, kBlock);
    const unsigned gf = grid_for(F, kBlock), gc = grid_for(C, kBlock);
    for (int sub = 0; sub < p->substeps; ++sub) {
        k_gravity<<<gv, kBlock, 0, s>>>(m->vertex, m->predicted_vertex, m->velocity, m->inverse_mass, g,
                                        p->velocity_dampening, p->dt, V);
        if ((fl & FFSRL_DISTANCE_XPBD) && E > 0) k_zero<<<ge, kBlock, 0, s>>>(m->edge_lambda, E);
        if ((fl & FFSRL_VOLUME_XPBD) && T > 0) k_zero<<<gt, kBlock, 0, s>>>(m->tetrahedron_lambda, T);
        for (int it = 0; it < p->iterations; ++it) {
            if ((fl & FFSRL_VOLUME) && T > 0)
                k_volume<<<gt, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number, m->tetrahedron,
                                               m->tetrahedron_rest_volume, m->inverse_mass, m->active_tetrahedron,
                                               p->ks_volume, T);
            if ((fl & FFSRL_VOLUME_XPBD) && T > 0)
                k_volume_xpbd<<<gt, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number,
                                                    m->tetrahedron_lambda, m->tetrahedron, m->xpbd_rest_volume,
                                                    m->inverse_mass, m->active_tetrahedron, avol, T);
            if ((fl & FFSRL_NEOHOOKEAN) && T > 0)
                k_neohookean<<<gt, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number, m->tetrahedron,
                                                   m->tetrahedron_rest_volume, m->inverse_mass, m->tetrahedron_dm_inv,
                                                   p->volume_compliance, p->deviatoric_compliance, p->dt, T);
            if ((fl & FFSRL_DISTANCE) && E > 0)
                k_distance<<<ge, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number, m->edge,
                                                 m->edge_rest_length, m->inverse_mass, m->active_edge, p->ks_distance,
                                                 E);
            if ((fl & FFSRL_DISTANCE_XPBD) && E > 0)
                k_distance_xpbd<<<ge, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number,
                                                      m->edge_lambda, m->edge, m->edge_rest_length, m->inverse_mass,
                                                      m->active_edge, adist, E);
            k_apply<<<gv, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number, V);
            if (fl & FFSRL_DRAG)
                k_drag<<<gv, kBlock, 0, s>>>(m->predicted_vertex, m->active_drag_constraint, m->vertex_to_env,
                                             m->laparoscope_tip, p->ks_drag, V);
            if ((fl & FFSRL_CONNECTORS) && C > 0)
                k_connector<<<gc, kBlock, 0, s>>>(m->predicted_vertex, m->dp, m->constraints_number,
                                                  m->connector_triangle_id, m->connector_tri_bar,
                                                  m->connector_vertex_id, m->connector_rest_dist,
                                                  p->connector_mass_weight_ratio, p->connector_ks,
                                                  p->connector_rest_length_mul, C);
            if ((fl & FFSRL_COLLIDE) && F > 0) {
                k_collide<<<gf, kBlock, 0, s>>>(m->predicted_vertex, m->collision_dp, m->triangle, m->tri_to_env,
                                                m->hole, m->inverse_mass, m->laparoscope_base, m->laparoscope_tip,
                                                m->laparoscope_radius, m->laparoscope_in_collision, p->ks_contact, F);
                k_collide_apply<<<gv, kBlock, 0, s>>>(m->predicted_vertex, m->collision_dp, V);
            }
        }
        k_bounds<<<gv, kBlock, 0, s>>>(m->predicted_vertex, p->ground_level, V);
        k_pbd<<<gv, kBlock, 0, s>>>(m->vertex, m->predicted_vertex, m->velocity, p->dt, V);
    }
    FFSRL_LAUNCH_CHECK("ffsrl_step_model");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_remap(float* dst, const float* src, const int32_t* map, int32_t count, void* stream) {
    if (count < 0 || (count > 0 && (!dst || !src || !map))) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_remap");
    if (count == 0) return FFSRL_OK;
    k_remap<<<grid_for(count, kBlock), kBlock, 0, (cudaStream_t)stream>>>(dst, src, map, count);
    FFSRL_LAUNCH_CHECK("ffsrl_remap");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_remap_envs(float* dst, const float* src, const int32_t* map, const int32_t* point_start,
                                    const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream) {
    if (n < 0 || num_envs < 0 || (n > 0 && (!dst || !src || !map || !point_start || !env_ids)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_remap_envs");
    if (n == 0) return FFSRL_OK;
    k_remap_envs<<<n, 256, 0, (cudaStream_t)stream>>>(dst, src, map, point_start, env_ids, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_remap_envs");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_update_clamps_drag(const float* positions, const int32_t* vertex_to_env,
                                            const float* laparoscope_tip, float* drag, float lookup_radius,
                                            const int32_t* state, const int32_t* update, int32_t num_vertices,
                                            void* stream) {
    if (num_vertices < 0 || (num_vertices > 0 && (!positions || !vertex_to_env || !laparoscope_tip || !drag ||
                                                  !state || !update)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_update_clamps_drag");
    if (num_vertices == 0) return FFSRL_OK;
    k_update_clamps<<<grid_for(num_vertices, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
        positions, vertex_to_env, laparoscope_tip, drag, lookup_radius, state, update, num_vertices);
    FFSRL_LAUNCH_CHECK("ffsrl_update_clamps_drag");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_force_clamps_drag(float* drag, int32_t vertex_id, const int32_t* env_id, int32_t num,
                                           float on, int32_t verts_per_env, void* stream) {
    if (num < 0 || (num > 0 && (!drag || !env_id))) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_force_clamps_drag");
    if (num == 0) return FFSRL_OK;
    k_force_clamps<<<grid_for(num, kBlock), kBlock, 0, (cudaStream_t)stream>>>(drag, vertex_id, env_id, on,
                                                                               verts_per_env, num);
    FFSRL_LAUNCH_CHECK("ffsrl_force_clamps_drag");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_grasp_nearest(const float* positions, const int32_t* cand_start, const int32_t* cand,
                                       const float* laparoscope_tip, const int32_t* clamp, float radius, float* drag,
                                       int32_t num_envs, void* stream) {
    if (num_envs < 0 || (num_envs > 0 && (!positions || !cand_start || !cand || !laparoscope_tip || !clamp || !drag)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_grasp_nearest");
    if (num_envs == 0) return FFSRL_OK;
    k_grasp_nearest<<<num_envs, 256, 0, (cudaStream_t)stream>>>(positions, cand_start, cand, laparoscope_tip, clamp,
                                                                radius, drag, nullptr, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_grasp_nearest");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_grasp_nearest_envs(const float* positions, const int32_t* cand_start, const int32_t* cand,
                                            const float* laparoscope_tip, const int32_t* clamp, float radius,
                                            float* drag, const int32_t* env_ids, int32_t n, int32_t num_envs,
                                            void* stream) {
    if (n < 0 || num_envs < 0 ||
        (n > 0 && (!positions || !cand_start || !cand || !laparoscope_tip || !clamp || !drag || !env_ids)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_grasp_nearest_envs");
    if (n == 0) return FFSRL_OK;
    k_grasp_nearest<<<n, 256, 0, (cudaStream_t)stream>>>(positions, cand_start, cand, laparoscope_tip, clamp, radius,
                                                         drag, env_ids, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_grasp_nearest_envs");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_move_tool_envs(float* laparoscope_base, float* laparoscope_tip, const float* disp,
                                        const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream) {
    if (n < 0 || num_envs < 0 || (n > 0 && (!laparoscope_base || !laparoscope_tip || !disp || !env_ids)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_move_tool_envs");
    if (n == 0) return FFSRL_OK;
    k_move_tool_envs<<<grid_for(4ll * n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(laparoscope_base, laparoscope_tip,
                                                                                    disp, env_ids, n, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_move_tool_envs");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_reset_envs(float* vertex, float* velocity, float* active_drag, const float* initial_vertex,
                                    float* laparoscope_base, float* laparoscope_tip, const float* initial_base,
                                    const float* initial_tip, int32_t* in_collision, float* xform,
                                    const float* initial_xform, const int32_t* env_vertex_start,
                                    const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream) {
    if (n < 0 || num_envs < 0 ||
        (n > 0 && (!vertex || !velocity || !active_drag || !initial_vertex || !laparoscope_base || !laparoscope_tip ||
                   !initial_base || !initial_tip || !in_collision || !env_vertex_start || !env_ids ||
                   (xform && !initial_xform))))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_reset_envs");
    if (n == 0) return FFSRL_OK;
    k_reset_envs<<<n, 256, 0, (cudaStream_t)stream>>>(vertex, velocity, active_drag, initial_vertex, laparoscope_base,
                                                       laparoscope_tip, initial_base, initial_tip, in_collision, xform,
                                                       initial_xform, env_vertex_start, env_ids, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_reset_envs");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_move_tool(float* laparoscope_base, float* laparoscope_tip, const float* disp,
                                   int32_t num_envs, void* stream) {
    if (num_envs < 0 || (num_envs > 0 && (!laparoscope_base || !laparoscope_tip || !disp)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_move_tool");
    if (num_envs == 0) return FFSRL_OK;
    k_move_tool<<<grid_for(4ll * num_envs, kBlock), kBlock, 0, (cudaStream_t)stream>>>(laparoscope_base,
                                                                                       laparoscope_tip, disp, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_move_tool");
    return FFSRL_OK;
}

// ---------------------------------------------------------------------------------
// Step without allocation.  Some callers cannot call cudaMalloc: a host application
// that has already reserved the device's memory for its own pool, or a control loop
// that must never wait on the driver's allocator.  For them this entry point runs the
// same step as ffsrl_step_model but keeps the three per-vertex accumulators that step
// needs (correction sum, contribution count, contact response) in one array compiled
// into the library, so the caller passes only the model's own inputs and outputs.
//
// Limits and rules:
//  - at most kNoAllocMaxVertices vertices per call (1.75 MB of device memory, held by
//    every GPU that loads the library until the process exits);
//  - the array is shared by every call: the first 28 bytes per vertex are cleared at the
//    start of each call, so nothing carries over between calls (ffsrl_step_model keeps
//    connector corrections made after the last apply for the next call; with
//    connectors, use ffsrl_step_model);
//  - calls whose work overlaps on the GPU (different streams, or different threads
//    without ordering) race on the array;
//  - the first call on a device looks up the array's device address (once per device,
//    with that device current); make that first call before any stream capture.
namespace {
constexpr int kNoAllocMaxVertices = 65536;
constexpr size_t kNoAllocBytesPerVertex = 28;  // dp (12) + collision dp (12) + count (4)
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocMaxVertices * kNoAllocBytesPerVertex];
constexpr int kMaxDevices = 256;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};
}  // namespace

extern "C" int32_t ffsrl_step_model_noalloc(const ffsrl_model* m, const ffsrl_params* p, void* stream) {
    if (!m || !p) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model_noalloc: null model or params");
    if (m->num_vertices < 0 || m->num_vertices > kNoAllocMaxVertices)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step_model_noalloc: " + std::to_string(m->num_vertices) +
                                                    " vertices exceed the limit of " +
                                                    std::to_string(kNoAllocMaxVertices));
    int dev = 0;
    FFSRL_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_step_model_noalloc: device ordinal");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            cudaError_t e = cudaGetSymbolAddress(&g_noalloc_addr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_addr[dev] = nullptr;
                return cuda_fail(e, "ffsrl_step_model_noalloc: cudaGetSymbolAddress");
            }
        }
        base = g_noalloc_addr[dev];
    }
    const size_t V = (size_t)m->num_vertices;
    unsigned char* s = static_cast<unsigned char*>(base);
    ffsrl_model mm = *m;
    mm.dp = reinterpret_cast<float*>(s);
    mm.collision_dp = reinterpret_cast<float*>(s + 12 * (size_t)kNoAllocMaxVertices);
    mm.constraints_number = reinterpret_cast<int32_t*>(s + 24 * (size_t)kNoAllocMaxVertices);
    cudaStream_t st = (cudaStream_t)stream;
    if (V > 0) {
        FFSRL_CUDA_TRY(cudaMemsetAsync(mm.dp, 0, 12 * V, st));
        FFSRL_CUDA_TRY(cudaMemsetAsync(mm.collision_dp, 0, 12 * V, st));
        FFSRL_CUDA_TRY(cudaMemsetAsync(mm.constraints_number, 0, 4 * V, st));
    }
    return ffsrl_step_model(&mm, p, stream);
}
