// instrument.cu -- laparoscope kinematics: the per-env transform hierarchy driven by RL
// actions, and the capsule ends the contact and grasp use (reference:
// FF_SRL/FF_SRL/modelDO.py:26-416, 1331-1419, 1552-1587; laparoscope.py:370-383).
//
// Each env owns 7 transforms, stored as the reference stores them (modelDO.py:1206): a
// 4x4 float matrix per slot, row-major, holding the transpose of the column-vector
// transform (p' = C p).  Slots: 0 rod capsule, 1 left clamp, 2 right clamp, 3 rotation
// centre (the trocar), 4 left-clamp pivot, 5 right-clamp pivot, 6 rod.  Moving a slot
// moves its children with it, keeping their pose relative to it:
//   0 -> 1 2 4 5 6,   3 -> 0 1 2 4 5 6,   4 -> 1,   5 -> 2.
//
// One thread per env does the whole update in a fixed order, then writes the env's four
// capsule ends (three capsules and the drag point).  The reference runs the rod, rotation
// centre and clamp actions as seven threads of one env writing the same matrices; the
// order here (rod, rotation centre, clamps) is the order a warp executes those branches
// in program order.
//
// This unit is compiled without FMA contraction; matrix products sum k = 0..3 in order.
// The reference's Warp built-ins (mat44 from translation/quaternion/scale, inverse,
// quat_from_axis_angle) are written from their mathematics.
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include "ffsrl_internal.h"

namespace ffsrl {
namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kClampMax = 85.0f, kClampMin = 40.0f, kClampDrag = 3.0f;  // degrees (modelDO.py:19-21)

struct M4 { float m[4][4]; };
struct F3 { float x, y, z; };

__device__ __forceinline__ F3 f3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len3(F3 a) { return sqrtf(dot3(a, a)); }

// slot s of an env: stored transpose -> column form, and back
__device__ __forceinline__ M4 load(const float* X, int s) {
    M4 c;
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) c.m[r][k] = X[16 * s + 4 * k + r];
    return c;
}
__device__ __forceinline__ void store(float* X, int s, const M4& c) {
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) X[16 * s + 4 * k + r] = c.m[r][k];
}

__device__ M4 mul(const M4& a, const M4& b) {
    M4 c;
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k)
            c.m[r][k] = ((a.m[r][0] * b.m[0][k] + a.m[r][1] * b.m[1][k]) + a.m[r][2] * b.m[2][k]) + a.m[r][3] * b.m[3][k];
    return c;
}

// general 4x4 inverse: adjugate over the determinant, the 2x2 minors of the top and
// bottom row pairs forming the cofactors (Laplace expansion along those row pairs)
__device__ M4 inverse(const M4& a) {
    const float(*m)[4] = a.m;
    float s0 = m[0][0] * m[1][1] - m[1][0] * m[0][1], s1 = m[0][0] * m[1][2] - m[1][0] * m[0][2];
    float s2 = m[0][0] * m[1][3] - m[1][0] * m[0][3], s3 = m[0][1] * m[1][2] - m[1][1] * m[0][2];
    float s4 = m[0][1] * m[1][3] - m[1][1] * m[0][3], s5 = m[0][2] * m[1][3] - m[1][2] * m[0][3];
    float c5 = m[2][2] * m[3][3] - m[3][2] * m[2][3], c4 = m[2][1] * m[3][3] - m[3][1] * m[2][3];
    float c3 = m[2][1] * m[3][2] - m[3][1] * m[2][2], c2 = m[2][0] * m[3][3] - m[3][0] * m[2][3];
    float c1 = m[2][0] * m[3][2] - m[3][0] * m[2][2], c0 = m[2][0] * m[3][1] - m[3][0] * m[2][1];
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    float inv = 1.0f / det;
    M4 b;
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

__device__ __forceinline__ F3 xform_point(const M4& c, F3 p) {
    return f3(((c.m[0][0] * p.x + c.m[0][1] * p.y) + c.m[0][2] * p.z) + c.m[0][3],
              ((c.m[1][0] * p.x + c.m[1][1] * p.y) + c.m[1][2] * p.z) + c.m[1][3],
              ((c.m[2][0] * p.x + c.m[2][1] * p.y) + c.m[2][2] * p.z) + c.m[2][3]);
}

// rigid transform from a translation and the rotation of the quaternion
// (axis sin(a/2), cos(a/2)); unit scale
__device__ M4 rigid(F3 t, F3 axis, float angle) {
    float h = 0.5f * angle;
    float s = sinf(h), w = cosf(h);
    float x = axis.x * s, y = axis.y * s, z = axis.z * s;
    M4 c;
    c.m[0][0] = 1.0f - 2.0f * (y * y + z * z); c.m[0][1] = 2.0f * (x * y - z * w); c.m[0][2] = 2.0f * (x * z + y * w);
    c.m[1][0] = 2.0f * (x * y + z * w); c.m[1][1] = 1.0f - 2.0f * (x * x + z * z); c.m[1][2] = 2.0f * (y * z - x * w);
    c.m[2][0] = 2.0f * (x * z - y * w); c.m[2][1] = 2.0f * (y * z + x * w); c.m[2][2] = 1.0f - 2.0f * (x * x + y * y);
    c.m[0][3] = t.x; c.m[1][3] = t.y; c.m[2][3] = t.z;
    c.m[3][0] = 0.0f; c.m[3][1] = 0.0f; c.m[3][2] = 0.0f; c.m[3][3] = 1.0f;
    return c;
}

// getTransformationMatrix (modelDO.py:396-414): T(shift) Rx(ax) Ry(ay) Rz(az)
__device__ M4 shift_rotate(float sx, float sy, float sz, float ax, float ay, float az) {
    const F3 zero = f3(0.0f, 0.0f, 0.0f);
    M4 T = rigid(f3(sx, sy, sz), zero, 0.0f);
    M4 X = rigid(zero, f3(1.0f, 0.0f, 0.0f), ax);
    M4 Y = rigid(zero, f3(0.0f, 1.0f, 0.0f), ay);
    M4 Z = rigid(zero, f3(0.0f, 0.0f, 1.0f), az);
    return mul(T, mul(X, mul(Y, Z)));
}

// applyTransformationToChild (modelDO.py:386-394): C' = P (M (P^-1 C)), P the parent now
__device__ void to_child(float* X, const M4& M, int parent, int child) {
    M4 P = load(X, parent);
    M4 C = load(X, child);
    store(X, child, mul(P, mul(M, mul(inverse(P), C))));
}

// applyTransformationToChildren (modelDO.py:366-384)
__device__ void to_children(float* X, const M4& M, int parent) {
    if (parent == 4) to_child(X, M, 4, 1);
    if (parent == 5) to_child(X, M, 5, 2);
    if (parent == 3)
        for (int i = 0; i < 7; ++i)
            if (i != 3) to_child(X, M, 3, i);
    if (parent == 0)
        for (int i = 1; i < 7; ++i)
            if (i != 3) to_child(X, M, 0, i);
}

// transformFunc (modelDO.py:291-298): children first, then the slot itself
__device__ void transform_slot(float* X, int slot, const M4& current, const M4& M) {
    to_children(X, M, slot);
    store(X, slot, mul(current, M));
}

// rotateClampsFunc (modelDO.py:300-364)
__device__ void rotate_clamps(float* X, int* dch, int* dchu, float action) {
    float diff = action * 180.0f / kPi;
    if (diff == 0.0f) return;
    M4 rod = load(X, 0);
    M4 left = load(X, 4);
    M4 right = load(X, 5);
    M4 local = mul(inverse(rod), right);
    float cur = asinf(local.m[2][1]) * 180.0f / kPi;
    bool apply = false;
    if (dch[0] == 1 && dchu[0] == 1) dchu[0] = 0;
    if (action > 0.0f) {
        if (cur < kClampMax) {
            if (cur + diff > kClampMax) diff = kClampMax - cur;
            apply = true;
        }
        if (cur > kClampDrag + kClampMin && dch[0] == 1) { dch[0] = 0; dchu[0] = 1; }
    } else {
        if (cur > kClampMin) {
            if (cur + diff < kClampMin) diff = kClampMin - cur;
            apply = true;
        }
        if (cur < kClampDrag + kClampMin && dch[0] == 0) { dch[0] = 1; dchu[0] = 1; }
    }
    if (apply) {
        float rad = diff * kPi / 180.0f;
        M4 R = shift_rotate(0.0f, 0.0f, 0.0f, rad, 0.0f, 0.0f);
        M4 Rinv = shift_rotate(0.0f, 0.0f, 0.0f, -rad, 0.0f, 0.0f);
        store(X, 4, mul(left, Rinv));
        to_children(X, Rinv, 4);
        store(X, 5, mul(right, R));
        to_children(X, R, 5);
    }
}

// updateLaparoscopeKernel (modelDO.py:222-245): capsule ends of rod and clamps, and the
// drag point as the tip of entry 3
__device__ void update_ends(const float* X, const float* height, float* base, float* tip, int e) {
    for (int k = 0; k < 4; ++k) {
        M4 c;
        F3 bl, tl;
        if (k < 3) {
            c = load(X, k);
            float h = height[4 * e + k];
            bl = f3(0.0f, 0.0f, 0.0f - h / 1.85f);
            tl = f3(0.0f, 0.0f, 0.0f + h / 1.85f);
        } else {
            c = load(X, 0);
            float rh = height[4 * e], ch = height[4 * e + 2];
            bl = f3(0.0f, 0.0f, 0.0f - rh * 0.5f - ch * 1.0f);
            tl = f3(0.0f, 0.0f, 0.0f + rh * 0.5f + ch * 1.0f);
        }
        F3 b = xform_point(c, bl), t = xform_point(c, tl);
        long long o = 3ll * (4 * e + k);
        base[o] = b.x; base[o + 1] = b.y; base[o + 2] = b.z;
        tip[o] = t.x; tip[o + 1] = t.y; tip[o + 2] = t.z;
    }
}

struct Kin {
    float* xform; float* base; float* tip; const float* height; int* dch; int* dchu; int num_envs;
};

// applyActionsKernel (modelDO.py:161-190): actions[5e..5e+4] = rod forward, rod roll,
// rotation-centre x and y, clamp opening
__global__ void k_apply_actions(Kin k, const float* __restrict__ actions) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= k.num_envs) return;
    float* X = k.xform + 112ll * e;
    const float* a = actions + 5ll * e;
    M4 rod0 = load(X, 0), rc0 = load(X, 3);  // each slot's own matrix as its thread reads it
    transform_slot(X, 0, rod0, shift_rotate(0.0f, 0.0f, a[0], 0.0f, 0.0f, a[1]));
    transform_slot(X, 3, rc0, shift_rotate(0.0f, 0.0f, 0.0f, a[2], a[3], 0.0f));
    rotate_clamps(X, k.dch + 3ll * e, k.dchu + 3ll * e, a[4]);
    update_ends(X, k.height, k.base, k.tip, e);
}

// transfromCartesianActionsKernel[InWorkspace] (modelDO.py:56-153): the effector moves
// by the action about the rotation centre -- a rotation of the instrument about the
// centre and a change of insertion depth.  With a workspace, components that would leave
// it are dropped and the env's violation flag is set.  With an env list, actions[3i..]
// move env ids[i] (ids outside [0, num_envs) skipped).
__global__ void k_cartesian(Kin k, const float* __restrict__ actions, int use_ws, float lx, float ly, float lz,
                            float hx, float hy, float hz, int* violation, const int* __restrict__ ids, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = ids ? ids[i] : i;
    if (e < 0 || e >= k.num_envs) return;
    const float* a = actions + 3ll * i;
    if (a[0] == 0.0f && a[1] == 0.0f && a[2] == 0.0f) return;
    float* X = k.xform + 112ll * e;
    const long long d = 3ll * (4 * e + 3);
    F3 cur = f3(k.tip[d], k.tip[d + 1], k.tip[d + 2]);
    F3 act = f3(a[0], a[1], a[2]);
    if (use_ws) {
        if (violation) violation[e] = 0;
        F3 nw = add(cur, act);
        if (nw.x < lx || nw.x > hx) { act.x = 0.0f; if (violation) violation[e] = 1; }
        if (nw.y < ly || nw.y > hy) { act.y = 0.0f; if (violation) violation[e] = 1; }
        if (nw.z < lz || nw.z > hz) { act.z = 0.0f; if (violation) violation[e] = 1; }
    }
    M4 rod = load(X, 0), rc = load(X, 3);
    F3 rel = xform_point(inverse(rc), cur);
    // the action in the centre's frame: the stored (transposed) matrix applied as a
    // column-form transform (modelDO.py:77) -- the transposed rotation
    F3 delta = f3(((rc.m[0][0] * act.x + rc.m[1][0] * act.y) + rc.m[2][0] * act.z) + rc.m[3][0],
                  ((rc.m[0][1] * act.x + rc.m[1][1] * act.y) + rc.m[2][1] * act.z) + rc.m[3][1],
                  ((rc.m[0][2] * act.x + rc.m[1][2] * act.y) + rc.m[2][2] * act.z) + rc.m[3][2]);
    F3 nrel = add(rel, delta);
    float rcur = len3(rel), rnew = len3(nrel);
    F3 cr = cross3(rel, nrel);
    float sin_t = len3(cr) / (len3(rel) * len3(nrel));
    float lc = len3(cr);
    F3 axis = lc > 0.0f ? f3(cr.x / lc, cr.y / lc, cr.z / lc) : f3(0.0f, 0.0f, 0.0f);
    float angle = asinf(sin_t);
    transform_slot(X, 0, rod, shift_rotate(0.0f, 0.0f, rnew - rcur, 0.0f, 0.0f, 0.0f));
    transform_slot(X, 3, rc, rigid(f3(0.0f, 0.0f, 0.0f), axis, angle));
    update_ends(X, k.height, k.base, k.tip, e);
}

// setRotationCenterTransformKernel (modelDO.py:155-171): the centre moves to the pose
// T(translation) Rx Ry Rz(rotation), carrying its children
__global__ void k_set_center(Kin k, const float* __restrict__ t, const float* __restrict__ r) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= k.num_envs) return;
    float* X = k.xform + 112ll * e;
    M4 rc = load(X, 3);
    const long long o = 3ll * e;
    M4 G = shift_rotate(t[o], t[o + 1], t[o + 2], r[o], r[o + 1], r[o + 2]);
    transform_slot(X, 3, rc, mul(inverse(rc), G));
    update_ends(X, k.height, k.base, k.tip, e);
}

__global__ void k_update_ends(Kin k) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= k.num_envs) return;
    update_ends(k.xform + 112ll * e, k.height, k.base, k.tip, e);
}

// updateLaparoscopeMeshKernel (modelDO.py:202-216) as transformSimLaparoscopeMeshData runs
// it (modelDO.py:1446-1473): one block per env stages the env's 7 transforms in shared
// memory; each thread carries local points (one instrument shape shared by every env)
// by the transform of their slot into the env's visual points
__global__ void k_visual(const float* __restrict__ xform, const float* __restrict__ local,
                         const int* __restrict__ slot, int num_points, float* __restrict__ vis,
                         const int* __restrict__ first, const int* __restrict__ ids, int num_envs) {
    const int e = ids ? ids[blockIdx.x] : blockIdx.x;
    if (e < 0 || e >= num_envs) return;
    __shared__ float X[112];
    for (int k = threadIdx.x; k < 112; k += blockDim.x) X[k] = xform[112ll * e + k];
    __syncthreads();
    const long long o = first[e];
    for (int i = threadIdx.x; i < num_points; i += blockDim.x) {
        const int s = slot[i];
        if (s < 0 || s > 6) continue;
        F3 p = xform_point(load(X, s), f3(local[3 * i], local[3 * i + 1], local[3 * i + 2]));
        float* q = vis + 3 * (o + i);
        q[0] = p.x; q[1] = p.y; q[2] = p.z;
    }
}

int32_t check_kin(const Kin& k, const char* what) {
    if (k.num_envs < 0 || (k.num_envs > 0 && (!k.xform || !k.base || !k.tip || !k.height)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, std::string(what) + ": null array or negative env count");
    return FFSRL_OK;
}

int32_t launch_cartesian(const Kin& k, const float* actions, const float* w, int32_t* violation, const int32_t* ids,
                         int32_t n, cudaStream_t s, const char* what) {
    k_cartesian<<<grid_for(n, 128), 128, 0, s>>>(k, actions, w ? 1 : 0, w ? w[0] : 0.0f, w ? w[1] : 0.0f,
                                                  w ? w[2] : 0.0f, w ? w[3] : 0.0f, w ? w[4] : 0.0f, w ? w[5] : 0.0f,
                                                  violation, ids, n);
    FFSRL_LAUNCH_CHECK(what);
    return FFSRL_OK;
}

}  // namespace
}  // namespace ffsrl

using namespace ffsrl;

extern "C" int32_t ffsrl_instrument_update(float* xform, float* base, float* tip, const float* height,
                                           int32_t num_envs, void* stream) {
    Kin k{xform, base, tip, height, nullptr, nullptr, num_envs};
    if (int32_t st = check_kin(k, "ffsrl_instrument_update")) return st;
    if (num_envs == 0) return FFSRL_OK;
    k_update_ends<<<grid_for(num_envs, 128), 128, 0, (cudaStream_t)stream>>>(k);
    FFSRL_LAUNCH_CHECK("ffsrl_instrument_update");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_instrument_apply_actions(float* xform, const float* actions, int32_t* drag_cut_heat,
                                                  int32_t* drag_cut_heat_update, float* base, float* tip,
                                                  const float* height, int32_t num_envs, void* stream) {
    Kin k{xform, base, tip, height, drag_cut_heat, drag_cut_heat_update, num_envs};
    if (int32_t st = check_kin(k, "ffsrl_instrument_apply_actions")) return st;
    if (num_envs > 0 && (!actions || !drag_cut_heat || !drag_cut_heat_update))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_instrument_apply_actions: null actions or clamp state");
    if (num_envs == 0) return FFSRL_OK;
    k_apply_actions<<<grid_for(num_envs, 128), 128, 0, (cudaStream_t)stream>>>(k, actions);
    FFSRL_LAUNCH_CHECK("ffsrl_instrument_apply_actions");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_instrument_cartesian(float* xform, const float* actions, const float* workspace,
                                              int32_t* violation, float* base, float* tip, const float* height,
                                              int32_t num_envs, void* stream) {
    Kin k{xform, base, tip, height, nullptr, nullptr, num_envs};
    if (int32_t st = check_kin(k, "ffsrl_instrument_cartesian")) return st;
    if (num_envs > 0 && !actions) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_instrument_cartesian: null actions");
    if (num_envs == 0) return FFSRL_OK;
    return launch_cartesian(k, actions, workspace, violation, nullptr, num_envs, (cudaStream_t)stream,
                            "ffsrl_instrument_cartesian");
}

extern "C" int32_t ffsrl_instrument_cartesian_envs(float* xform, const float* actions, const float* workspace,
                                                   int32_t* violation, float* base, float* tip, const float* height,
                                                   const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream) {
    Kin k{xform, base, tip, height, nullptr, nullptr, num_envs};
    if (int32_t st = check_kin(k, "ffsrl_instrument_cartesian_envs")) return st;
    if (n < 0 || (n > 0 && (!actions || !env_ids)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_instrument_cartesian_envs: null actions or ids");
    if (n == 0) return FFSRL_OK;
    return launch_cartesian(k, actions, workspace, violation, env_ids, n, (cudaStream_t)stream,
                            "ffsrl_instrument_cartesian_envs");
}

extern "C" int32_t ffsrl_instrument_set_rotation_center(float* xform, const float* translation,
                                                        const float* rotation, float* base, float* tip,
                                                        const float* height, int32_t num_envs, void* stream) {
    Kin k{xform, base, tip, height, nullptr, nullptr, num_envs};
    if (int32_t st = check_kin(k, "ffsrl_instrument_set_rotation_center")) return st;
    if (num_envs > 0 && (!translation || !rotation))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_instrument_set_rotation_center: null pose");
    if (num_envs == 0) return FFSRL_OK;
    k_set_center<<<grid_for(num_envs, 128), 128, 0, (cudaStream_t)stream>>>(k, translation, rotation);
    FFSRL_LAUNCH_CHECK("ffsrl_instrument_set_rotation_center");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_instrument_visual_update(const float* xform, const float* local_point,
                                                  const int32_t* point_slot, int32_t num_points, float* vis_point,
                                                  const int32_t* env_first_point, const int32_t* env_ids, int32_t n,
                                                  int32_t num_envs, void* stream) {
    if (n < 0 || num_points < 0 || num_envs < 0 || (!env_ids && n != num_envs))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_instrument_visual_update: bad counts");
    if (n == 0 || num_points == 0) return FFSRL_OK;
    if (!xform || !local_point || !point_slot || !vis_point || !env_first_point)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_instrument_visual_update: null array");
    k_visual<<<n, 128, 0, (cudaStream_t)stream>>>(xform, local_point, point_slot, num_points, vis_point,
                                                  env_first_point, env_ids, num_envs);
    FFSRL_LAUNCH_CHECK("ffsrl_instrument_visual_update");
    return FFSRL_OK;
}
