// render.cu -- BVH refit and ray-cast renderer (reference: FF_SRL/FF_SRL/bvh.py:30-104,
// 419-454 and render.py:81-121, 276-498, 588-724, 975-1022).
//
// This unit is compiled with -fmad=false: every product and sum rounds as written, so
// with IEEE division and square root the images and boxes equal the CPU restatement's
// bit for bit whenever the summation order is the same (the fused paths).
#include <cuda_runtime.h>
#include <cstdint>
#include "ffsrl_internal.h"
#include "vecmath.cuh"

namespace ffsrl {
namespace {

constexpr int kStackCap = 64;  // traversal stack entries per ray (the reference uses 32)

__device__ __forceinline__ int find_env(const int* __restrict__ node_offset, int n_env, int total, int tid) {
    // env whose AABB range [node_offset[e], next) holds tid; node_offset ascending
    int lo = 0, hi = n_env - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (node_offset[mid] <= tid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void refit_node(const ffsrl_bvh& b, const float* __restrict__ pts,
                                           const int* __restrict__ faces, int e, int n0, int t0, int base, int node) {
    int left = b.left_node[n0 + node];
    v3 lo, hi;
    if (left < 0) {
        lo = mk(1e6f, 1e6f, 1e6f);
        hi = mk(-1e6f, -1e6f, -1e6f);
        int first = b.first_tri_id[n0 + node];
        int cnt = b.tri_count[n0 + node];
        long long fofs = b.env_face_offset[e];
        for (int k = 0; k < cnt; ++k) {
            long long f = fofs + b.tri_id[t0 + first + k];
            // the reference's refit may box another face than the one it traverses
            // (bvh.py:66-74 against render.py:462-470); refit_source holds that face
            const long long fb = b.refit_source ? (long long)b.refit_source[f] : f;
            v3 pA = ld3(pts, faces[3 * fb]), pB = ld3(pts, faces[3 * fb + 1]), pC = ld3(pts, faces[3 * fb + 2]);
            lo = vmin(pA, vmin(pB, vmin(pC, lo)));
            hi = vmax(pA, vmax(pB, vmax(pC, hi)));
            if (fb != f) pA = ld3(pts, faces[3 * f]), pB = ld3(pts, faces[3 * f + 1]), pC = ld3(pts, faces[3 * f + 2]);
            if (b.tri_pos) {
                float4* q = reinterpret_cast<float4*>(b.tri_pos) + 3 * (fofs + first + k);
                q[0] = make_float4(pA.x, pA.y, pA.z, pB.x);
                q[1] = make_float4(pB.y, pB.z, pC.x, pC.y);
                q[2] = make_float4(pC.z, 0.0f, 0.0f, 0.0f);
            }
        }
        if (b.node_box) {
            float4* nb = reinterpret_cast<float4*>(b.node_box) + 2ll * (base + node);
            nb[0] = make_float4(lo.x, lo.y, lo.z, __int_as_float(-1));
            nb[1] = make_float4(hi.x, hi.y, hi.z, __int_as_float(first * 256 + (cnt < 255 ? cnt : 255)));
        }
    } else {
        v3 l0 = ld3(b.aabb_min, base + left), h0 = ld3(b.aabb_max, base + left);
        v3 l1 = ld3(b.aabb_min, base + left + 1), h1 = ld3(b.aabb_max, base + left + 1);
        lo = vmin(l0, l1);
        hi = vmax(h0, h1);
        if (b.node_box) {
            // the traversal's child order: the axis along which the children's centres lie
            // farthest apart (bits 0-1) and whether the right child's centre is the higher
            // one (bit 2)
            const v3 d = (l1 + h1) - (l0 + h0);
            const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
            const int axis = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
            const float da = axis == 0 ? d.x : (axis == 1 ? d.y : d.z);
            float4* nb = reinterpret_cast<float4*>(b.node_box) + 2ll * (base + node);
            nb[0] = make_float4(lo.x, lo.y, lo.z, __int_as_float(left));
            nb[1] = make_float4(hi.x, hi.y, hi.z, __int_as_float(axis | (da > 0.0f ? 4 : 0)));
        }
    }
    st3(b.aabb_min, base + node, lo);
    st3(b.aabb_max, base + node, hi);
}

// refitBVHLevel (bvh.py:30-104): every env node at `level`
__global__ void k_refit_level(ffsrl_bvh b, const float* __restrict__ pts, const int* __restrict__ faces, int level) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= b.total_env_nodes) return;
    int e = find_env(b.env_node_offset, b.num_envs, b.total_env_nodes, tid);
    int topo = b.env_topology[e];
    int n0 = b.topo_node_offset[topo];
    int node = tid - b.env_node_offset[e];
    if (node >= b.topo_node_offset[topo + 1] - n0) return;
    if (b.level[n0 + node] != level) return;
    refit_node(b, pts, faces, e, n0, b.topo_tri_offset[topo], b.env_node_offset[e], node);
}

// One block per env (or per listed env): levels deepest first, nodes of a level in parallel.
__global__ void k_refit_fused(ffsrl_bvh b, const float* __restrict__ pts, const int* __restrict__ faces,
                              const int* __restrict__ ids) {
    int e = ids ? ids[blockIdx.x] : blockIdx.x;
    if (e < 0 || e >= b.num_envs) return;
    int topo = b.env_topology[e];
    int n0 = b.topo_node_offset[topo], t0 = b.topo_tri_offset[topo];
    int base = b.env_node_offset[e];
    int lo = b.topo_level_offset[topo];
    int groups = b.topo_max_level[topo] + 1;
    for (int g = 0; g < groups; ++g) {
        int s0 = b.level_start[lo + g], s1 = b.level_start[lo + g + 1];
        for (int k = s0 + threadIdx.x; k < s1; k += blockDim.x) refit_node(b, pts, faces, e, n0, t0, base, b.level_node[k]);
        __syncthreads();
    }
}

__global__ void k_zero3(float* p, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3(p, i, mk(0.0f, 0.0f, 0.0f));
}

// vertex_normal_sum_kernel (render.py:81-105)
__global__ void k_normal_sum(const float* __restrict__ pts, const int* __restrict__ faces, float* nsum, int nf) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int i = faces[3 * f], j = faces[3 * f + 1], k = faces[3 * f + 2];
    v3 a = ld3(pts, i), b = ld3(pts, j), c = ld3(pts, k);
    v3 an = cross(b - a, c - a);
    atomic_add3(nsum, i, an); atomic_add3(nsum, j, an); atomic_add3(nsum, k, an);
}

// normalize_kernel (render.py:113-121)
__global__ void k_normalize(const float* __restrict__ nsum, float* __restrict__ nrm, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3(nrm, i, normalize(ld3(nsum, i)));
}

// Area-weighted normals gathered per point in ascending face order (deterministic; the
// same order as a serial run of vertex_normal_sum_kernel), then normalised.
__global__ void k_normal_gather(const float* __restrict__ pts, const int* __restrict__ faces,
                                const int* __restrict__ start, const int* __restrict__ pf, float* __restrict__ nrm,
                                int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 s = mk(0.0f, 0.0f, 0.0f);
    for (int k = start[i]; k < start[i + 1]; ++k) {
        long long f = pf[k];
        v3 a = ld3(pts, faces[3 * f]), b = ld3(pts, faces[3 * f + 1]), c = ld3(pts, faces[3 * f + 2]);
        s = s + cross(b - a, c - a);
    }
    st3(nrm, i, normalize(s));
}

// the same gather for the points of one listed env per block
__global__ void k_normal_gather_envs(const float* __restrict__ pts, const int* __restrict__ faces,
                                     const int* __restrict__ start, const int* __restrict__ pf, float* __restrict__ nrm,
                                     const int* __restrict__ pstart, const int* __restrict__ ids, int num_envs) {
    int e = ids[blockIdx.x];
    if (e < 0 || e >= num_envs) return;
    for (int i = pstart[e] + threadIdx.x; i < pstart[e + 1]; i += blockDim.x) {
        v3 s = mk(0.0f, 0.0f, 0.0f);
        for (int k = start[i]; k < start[i + 1]; ++k) {
            long long f = pf[k];
            v3 a = ld3(pts, faces[3 * f]), b = ld3(pts, faces[3 * f + 1]), c = ld3(pts, faces[3 * f + 2]);
            s = s + cross(b - a, c - a);
        }
        st3(nrm, i, normalize(s));
    }
}

__device__ __forceinline__ v3 quat_rotate(float4 q, v3 x) {
    v3 u = mk(q.x, q.y, q.z);
    float c = 2.0f * q.w * q.w - 1.0f;
    float d = 2.0f * (u.x * x.x + u.y * x.y + u.z * x.z);
    return x * c + u * d + cross(u, x) * (q.w * 2.0f);
}

// intersectAABB (render.py:588-609)
__device__ __forceinline__ bool slab(v3 ro, v3 rd, v3 lo, v3 hi, float& tnear) {
    float t1 = (lo.x - ro.x) / rd.x, t2 = (hi.x - ro.x) / rd.x;
    float t3 = (lo.y - ro.y) / rd.y, t4 = (hi.y - ro.y) / rd.y;
    float t5 = (lo.z - ro.z) / rd.z, t6 = (hi.z - ro.z) / rd.z;
    float tmin = fmax_ref(fmax_ref(fmin_ref(t1, t2), fmin_ref(t3, t4)), fmin_ref(t5, t6));
    float tmax = fmin_ref(fmin_ref(fmax_ref(t1, t2), fmax_ref(t3, t4)), fmax_ref(t5, t6));
    tnear = tmin;
    return (tmax >= 0.0f) && (tmax >= tmin);
}

// Node test of the traversal: intersectAABB's hit && tmin < tMin (render.py:452-454).
// The slab distances are first formed as fma(lo, inv, -ro inv) with the ray's reciprocal
// direction inv and the per-ray products ro inv.  Against the reference's
// (lo - ro) / rd each differs by at most 4.01 u |t| + 1.02 u |ro inv| (u = 2^-24: the
// reciprocal, the product ro inv and the fma each round once; the reference rounds the
// difference and the quotient).  When every part of the decision is farther from its
// threshold than that -- g = 8 u m + 4 u R below, m the sum of the six |t|, R the sum
// of the three |ro inv| -- the decision equals the reference's.  Otherwise, and for
// non-finite distances, the reference's divisions decide.
struct RaySlab {
    v3 inv;    // 1 / rd per axis
    v3 roinv;  // ro * inv per axis
    float g0;  // 4 u (|ro inv|.x + .y + .z)
};

__device__ __forceinline__ RaySlab ray_slab(v3 ro, v3 rd) {
    RaySlab r;
    r.inv = mk(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
    r.roinv = mk(ro.x * r.inv.x, ro.y * r.inv.y, ro.z * r.inv.z);
    r.g0 = 2.38418579e-7f * ((fabsf(r.roinv.x) + fabsf(r.roinv.y)) + fabsf(r.roinv.z));  // 4 * 2^-24
    return r;
}

__device__ __forceinline__ bool node_hit(v3 ro, v3 rd, const RaySlab& rs, v3 lo, v3 hi, float tMin) {
    float t1 = fmaf(lo.x, rs.inv.x, -rs.roinv.x), t2 = fmaf(hi.x, rs.inv.x, -rs.roinv.x);
    float t3 = fmaf(lo.y, rs.inv.y, -rs.roinv.y), t4 = fmaf(hi.y, rs.inv.y, -rs.roinv.y);
    float t5 = fmaf(lo.z, rs.inv.z, -rs.roinv.z), t6 = fmaf(hi.z, rs.inv.z, -rs.roinv.z);
    // the sum of magnitudes bounds every distance and is infinite or NaN when any of them
    // is (or when the per-ray products are), so the fast path only sees finite values,
    // where fminf/fmaxf pick what the reference's comparisons pick (up to the sign of a
    // zero, which no test below sees)
    float m = ((fabsf(t1) + fabsf(t2)) + (fabsf(t3) + fabsf(t4))) + (fabsf(t5) + fabsf(t6));
    if (m < 3.0e37f && rs.g0 < 3.0e37f) {
        float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
        float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
        float g = fmaf(m, 4.76837158e-7f, rs.g0);  // 8 u m + 4 u R
        // a certainly-false part decides a miss; all parts certainly true decide a hit
        if (tmax < -g || tmax - tmin < -2.0f * g || tmin > tMin + g) return false;
        if (tmax > g && tmax - tmin > 2.0f * g && tmin < tMin - g) return true;
    }
    float tn;
    bool h = slab(ro, rd, lo, hi, tn);
    return h && tn < tMin;
}

// MTTriRayIntersection (render.py:661-697)
__device__ __forceinline__ float moller_trumbore(v3 a, v3 b, v3 c, v3 ro, v3 rd, v3& p) {
    v3 ab = b - a, ac = c - a;
    v3 pvec = cross(rd, ac);
    float det = dot(ab, pvec);
    if (fabsf(det) < 0.0001f) return -1.0f;
    float invDet = 1.0f / det;
    v3 tvec = ro - a;
    float u = dot(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    v3 qvec = cross(tvec, ab);
    float v = dot(rd, qvec) * invDet;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    float t = dot(ac, qvec) * invDet;
    p = ro + t * rd;
    return t;
}

struct EnvView {
    const int* left; const int* first; const int* count; const int* tri;
    const float* amin; const float* amax;
    const float4* box;   // packed node boxes of the env (or null)
    const float4* tpos;  // leaf triangles of the env in tri-map order, 3 float4 each (or null)
    long long fofs;
    int nn;  // nodes in the topology
};

__device__ __forceinline__ EnvView env_view(const ffsrl_bvh& b, int e) {
    int topo = b.env_topology[e];
    EnvView v;
    int n0 = b.topo_node_offset[topo];
    v.left = b.left_node + n0; v.first = b.first_tri_id + n0; v.count = b.tri_count + n0;
    v.tri = b.tri_id + b.topo_tri_offset[topo];
    long long base = b.env_node_offset[e];
    v.amin = b.aabb_min + 3 * base; v.amax = b.aabb_max + 3 * base;
    v.fofs = b.env_face_offset[e];
    v.nn = b.topo_node_offset[topo + 1] - n0;
    v.box = b.node_box ? reinterpret_cast<const float4*>(b.node_box) + 2 * base : nullptr;
    v.tpos = b.tri_pos ? reinterpret_cast<const float4*>(b.tri_pos) + 3 * v.fofs : nullptr;
    return v;
}

// meshQueryRayManyEnvs (render.py:411-498) over the packed copies written by the refit
// (two 16-byte loads per node, contiguous leaf triangles), visiting the nearer child
// first: the refit stores per inner node the axis along which its children's centres lie
// farthest apart, and the ray's sign along it picks the order.  The result is the
// reference's hit.  The reference visits nodes in a fixed pre-order (right child first),
// prunes a node whose box entry is not nearer than the best hit so far, and keeps the
// first of equally near hits.  Its pre-order visits leaves in descending tri-map position
// (the build puts a node's left child's triangles first) and a leaf's triangles in
// ascending order.  So here a hit is kept when it is nearer, or equally near and earlier
// in that order.  With the same strict pruning, the triangle the reference keeps is never
// pruned, whatever the visiting order: its boxes are entered before it is reached.
// Returns the global face id or -1.
__device__ int query_packed(const EnvView& ev, v3 ro, v3 rd, float& t_hit, v3& p_hit, int* err) {
    int stack[kStackCap];
    int count = 1;
    stack[0] = 0;
    float tMin = 1e6f;
    int hit_tri = -1;
    int best_first = -1, best_k = 0;  // the kept hit's leaf and place in it
    int visits = 0;
    const RaySlab rs = ray_slab(ro, rd);
    while (count) {
        int node = stack[--count];
        if (++visits > ev.nn) {
            atomicExch(err, FFSRL_ERR_STACK_OVERFLOW);
            return -1;
        }
        const float4 a = __ldg(ev.box + 2 * node), c = __ldg(ev.box + 2 * node + 1);
        if (node_hit(ro, rd, rs, mk(a.x, a.y, a.z), mk(c.x, c.y, c.z), tMin)) {
            int left = __float_as_int(a.w);
            if (left == -1) {
                int fc = __float_as_int(c.w);
                int first = fc >> 8, cnt = fc & 255;
                if (cnt == 255) cnt = ev.count[node];
                for (int k = 0; k < cnt; ++k) {
                    const float4* q = ev.tpos + 3ll * (first + k);
                    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
                    v3 A = mk(q0.x, q0.y, q0.z);
                    v3 B = mk(q0.w, q1.x, q1.y);
                    v3 C = mk(q1.z, q1.w, q2.x);
                    v3 p;
                    float t = moller_trumbore(A, B, C, ro, rd, p);
                    if (t > 0.0f && (t < tMin || (t == tMin && hit_tri >= 0 &&
                                                  (first > best_first || (first == best_first && k < best_k))))) {
                        tMin = t;
                        hit_tri = (int)(ev.fofs + ev.tri[first + k]);
                        best_first = first;
                        best_k = k;
                        t_hit = t;
                        p_hit = p;
                    }
                }
            } else {
                if (left < 0 || left + 1 >= ev.nn) {
                    atomicExch(err, FFSRL_ERR_INVALID_ARGUMENT);
                    return -1;
                }
                if (count + 2 > kStackCap) {
                    atomicExch(err, FFSRL_ERR_STACK_OVERFLOW);
                    return -1;
                }
                const int code = __float_as_int(c.w);
                const int axis = code & 3;
                const float da = axis == 0 ? rd.x : (axis == 1 ? rd.y : rd.z);
                // nearer child: the left one when the ray runs towards the right child's side
                const bool left_near = (da > 0.0f) == ((code & 4) != 0);
                stack[count] = left_near ? left + 1 : left;
                stack[count + 1] = left_near ? left : left + 1;
                count += 2;
            }
        }
    }
    if (tMin >= 1e6f) hit_tri = -1;
    return hit_tri;
}

__device__ int query(const EnvView& ev, const float* __restrict__ pts, const int* __restrict__ faces, v3 ro, v3 rd,
                     float& t_hit, v3& p_hit, int* err) {
    if (ev.box && ev.tpos) return query_packed(ev, ro, rd, t_hit, p_hit, err);
    int stack[kStackCap];
    int count = 1;
    stack[0] = 0;
    float tMin = 1e6f;
    int hit_tri = -1;
    int visits = 0;
    const RaySlab rs = ray_slab(ro, rd);
    while (count) {
        int node = stack[--count];
        if (++visits > ev.nn) {  // a valid tree visits each node at most once
            atomicExch(err, FFSRL_ERR_STACK_OVERFLOW);
            return -1;
        }
        if (node_hit(ro, rd, rs, ld3(ev.amin, node), ld3(ev.amax, node), tMin)) {
            int left = ev.left[node];
            if (left == -1) {
                int first = ev.first[node];
                int cnt = ev.count[node];
                for (int k = 0; k < cnt; ++k) {
                    long long f = ev.fofs + ev.tri[first + k];
                    v3 A = ld3(pts, faces[3 * f]), B = ld3(pts, faces[3 * f + 1]), C = ld3(pts, faces[3 * f + 2]);
                    v3 p;
                    float t = moller_trumbore(A, B, C, ro, rd, p);
                    if (t < tMin && t > 0.0f) {
                        tMin = t;
                        hit_tri = (int)f; t_hit = t; p_hit = p;
                    }
                }
            } else {
                if (left < 0 || left + 1 >= ev.nn) {
                    atomicExch(err, FFSRL_ERR_INVALID_ARGUMENT);
                    return -1;
                }
                if (count + 2 > kStackCap) {
                    atomicExch(err, FFSRL_ERR_STACK_OVERFLOW);
                    return -1;
                }
                stack[count] = left;
                stack[count + 1] = left + 1;
                count += 2;
            }
        }
    }
    if (tMin >= 1e6f) hit_tri = -1;
    return hit_tri;
}

struct Shade { v3 color; float depth; };

// shading of drawSimBVHKernelManyEnvs (render.py:334-409): modes 0 grayscale, 1 texture,
// 2 normal map, 3 vertex colour, 4 depth map into `color`; `depth` gets t/50 in every mode
// The object of env e that holds env-local face lf (render.py:360-366: visFaceToObjectId,
// objectUsesTexture, objectNumVisFaceCummulative): its 5-int entry in object_texture.
__device__ __forceinline__ const int* face_object(const ffsrl_render& r, int e, int lf) {
    const int o0 = r.env_objects[2ll * e], no = r.env_objects[2ll * e + 1];
    const int* ob = r.object_texture + 5ll * o0;
    for (int k = 1; k < no; ++k) {
        if (r.object_texture[5ll * (o0 + k)] > lf) break;
        ob = r.object_texture + 5ll * (o0 + k);
    }
    return ob;
}

// texture_interpolation (render.py:123-148): bilinear texel of the interpolated tex
// coordinate; texel (x, y) of a texture at first + y + x*S.  Indices are clamped into the
// texture (the reference reads one texel past the edge at coordinate 1, weighted 0).
__device__ __forceinline__ v3 texel(const ffsrl_render& r, const int* ob, int lf, float u, float v, float w) {
    const int first = ob[1], S = ob[2], c0 = ob[3];
    const int* ti = r.tex_indices + ob[4] + 3ll * (lf - ob[0]);
    const float* ta = r.tex_coords + 2ll * (c0 + ti[0]);
    const float* tb = r.tex_coords + 2ll * (c0 + ti[1]);
    const float* tc = r.tex_coords + 2ll * (c0 + ti[2]);
    float tx = (u * ta[0] + v * tb[0]) + w * tc[0];
    float ty = (u * ta[1] + v * tb[1]) + w * tc[1];
    float fx = tx * float(S - 1), fy = (1.0f - ty) * float(S - 1);
    int x0 = (int)fx, y0 = (int)fy;
    float ax = fx - float(x0), ay = fy - float(y0);
    int x1 = x0 + 1, y1 = y0 + 1;
    x0 = min(max(x0, 0), S - 1); x1 = min(max(x1, 0), S - 1);
    y0 = min(max(y0, 0), S - 1); y1 = min(max(y1, 0), S - 1);
    v3 c00 = ld3(r.texture, (long long)first + y0 + x0 * S), c10 = ld3(r.texture, (long long)first + y0 + x1 * S);
    v3 c01 = ld3(r.texture, (long long)first + y1 + x0 * S), c11 = ld3(r.texture, (long long)first + y1 + x1 * S);
    v3 lower = (1.0f - ax) * c00 + ax * c10;
    v3 upper = (1.0f - ax) * c01 + ax * c11;
    return (1.0f - ay) * lower + ay * upper;
}

__device__ __forceinline__ Shade trace(const ffsrl_render& r, const EnvView& ev, int e, v3 ro, float4 q, int x, int y,
                                       int W, int H) {
    float sx = 2.0f * float(x) / float(W) - 1.0f;
    float sy = 2.0f * float(y) / float(H) - 1.0f;
    v3 rd = normalize(quat_rotate(q, mk(sx * r.camera_tan * r.camera_aspect, sy * r.camera_tan, -1.0f)));
    float t = 0.0f;
    v3 p = mk(0.0f, 0.0f, 0.0f);
    int tri = query(ev, r.vis_point, r.vis_face, ro, rd, t, p, r.error_flag);
    Shade s;
    s.color = mk(0.0f, 0.0f, 0.0f);
    s.depth = 0.0f;
    if (tri > -1) {
        int i = r.vis_face[3ll * tri], j = r.vis_face[3ll * tri + 1], k = r.vis_face[3ll * tri + 2];
        v3 a = ld3(r.vis_point, i), b = ld3(r.vis_point, j), c = ld3(r.vis_point, k);
        float area = length(cross(b - a, c - a));
        float w = length(cross(b - a, p - a)) / area;
        float v = length(cross(p - a, c - a)) / area;
        float u = 1.0f - w - v;
        v3 n = u * ld3(r.vertex_normal, i) + v * ld3(r.vertex_normal, j) + w * ld3(r.vertex_normal, k);
        v3 col;
        if (r.render_mode == 2) {  // normal map
            col = n * 0.5f + mk(0.5f, 0.5f, 0.5f);
        } else if (r.render_mode == 4) {  // depth map
            float g = t / 50.0f;
            col = mk(g, g, g);
        } else {
            v3 base;
            if (r.render_mode == 0)
                base = mk(1.0f, 1.0f, 1.0f);
            else {
                const int lf = (int)(tri - ev.fofs);
                const int* ob = (r.render_mode == 1 && r.env_objects) ? face_object(r, e, lf) : nullptr;
                if (ob && ob[2] > 0)
                    base = texel(r, ob, lf, u, v, w);
                else
                    base = (ld3(r.vis_point_color, i) + ld3(r.vis_point_color, j) + ld3(r.vis_point_color, k)) / 3.0f;
            }
            float lam = 0.0f;
            for (int l = 0; l < r.num_lights; ++l) {
                float val = r.light_intensity[l] * dot(n, ld3(r.light_dir, l));
                if (val < 0.0f) val = 0.0f;
                lam = lam + val;
            }
            col = lam * base;
        }
        if (col.x > 1.0f) col.x = 1.0f;
        if (col.y > 1.0f) col.y = 1.0f;
        if (col.z > 1.0f) col.z = 1.0f;
        s.color = col;
        float d = t / 50.0f;
        if (d > 1.0f) d = 1.0f;
        s.depth = d;
    }
    return s;
}

// drawSimBVHKernelManyEnvs (render.py:276-409): one thread per ray, into scratch
__global__ void k_draw(ffsrl_render r, ffsrl_bvh b) {
    const int W = 2 * r.resolution, H = 2 * r.resolution;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)W * H * r.num_envs) return;
    int e = (int)(tid / (W * H));
    int et = (int)(tid % (W * H));
    int x = et % W;
    int y = H - et / W;
    int cam = r.num_cameras > 1 ? e : 0;
    v3 ro = ld3(r.camera_pos, cam);
    float4 q = reinterpret_cast<const float4*>(r.camera_rot)[cam];
    EnvView ev = env_view(b, e);
    Shade s = trace(r, ev, e, ro, q, x, y, W, H);
    st3(r.rays, tid, s.color);
    r.ray_depth[tid] = s.depth;
}

// downsample_kernel (render.py:699-724), 2x2 rays per pixel
__global__ void k_downsample(ffsrl_render r) {
    const int R = r.resolution, W = 2 * R;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)R * R * r.num_envs) return;
    long long px = tid % R, py = tid / R;
    long long start = py * 2 * W + px * 2;
    v3 c = mk(0.0f, 0.0f, 0.0f);
    float d = 0.0f;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            v3 s = ld3(r.rays, start + i * W + j);
            c = mk(c.x + s.x, c.y + s.y, c.z + s.z);
            d = d + r.ray_depth[start + i * W + j];
        }
    float nsq = float(2 * 2);
    if (r.color) st3(r.color, tid, mk(c.x / nsq, c.y / nsq, c.z / nsq));
    if (r.depth) r.depth[tid] = d / nsq;
}

// One thread per ray; the four rays of a pixel sit in consecutive lanes and are summed
// by shuffles in downsample_kernel's order ((r00 + r01) + r10) + r11, then divided by 4.
// A block covers an 8x8 pixel tile of one env so neighbouring rays share BVH nodes in L1,
// and a warp's rays cover a compact 4x2-pixel patch (3% faster than a row of 8 pixels:
// closer rays take more of the same nodes).
__global__ void __launch_bounds__(256) k_rays(ffsrl_render r, ffsrl_bvh b, const int* __restrict__ ids, int n_ids) {
    const int R = r.resolution, W = 2 * R, H = 2 * R;
    const int tiles_x = (R + 7) / 8;
    const int tiles = tiles_x * ((R + 7) / 8);
    const int k = blockIdx.x / tiles;
    const int e = ids ? (k < n_ids ? ids[k] : r.num_envs) : k;
    const int tile = blockIdx.x % tiles;
    const int pix = threadIdx.x >> 2, q = threadIdx.x & 3;
    // a warp's eight pixels form a 4x2 patch; the tile's eight warps form 2x4 patches
    const int wp = pix >> 3, j = pix & 7;
    const int px = (tile % tiles_x) * 8 + (wp & 1) * 4 + (j & 3);
    const int py = (tile / tiles_x) * 8 + (wp >> 1) * 2 + (j >> 2);
    const bool valid = e >= 0 && e < r.num_envs && px < R && py < R;
    Shade s;
    s.color = mk(0.0f, 0.0f, 0.0f);
    s.depth = 0.0f;
    if (valid) {
        const int cam = r.num_cameras > 1 ? e : 0;
        const v3 ro = ld3(r.camera_pos, cam);
        const float4 qr = reinterpret_cast<const float4*>(r.camera_rot)[cam];
        const EnvView ev = env_view(b, e);
        const int et = (2 * py + (q >> 1)) * W + 2 * px + (q & 1);  // ray index as in downsample_kernel
        s = trace(r, ev, e, ro, qr, et % W, H - et / W, W, H);
    }
    float cx = s.color.x, cy = s.color.y, cz = s.color.z, d = s.depth;
    float ax[3], ay[3], az[3], ad[3];
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
        ax[k - 1] = __shfl_down_sync(0xffffffffu, cx, k);
        ay[k - 1] = __shfl_down_sync(0xffffffffu, cy, k);
        az[k - 1] = __shfl_down_sync(0xffffffffu, cz, k);
        ad[k - 1] = __shfl_down_sync(0xffffffffu, d, k);
    }
    if (valid && q == 0) {
        v3 c = mk(cx, cy, cz);
        for (int k = 0; k < 3; ++k) c = mk(c.x + ax[k], c.y + ay[k], c.z + az[k]);
        float dd = ((d + ad[0]) + ad[1]) + ad[2];
        float nsq = float(2 * 2);
        long long o = (long long)e * R * R + (long long)py * R + px;
        if (r.color) st3(r.color, o, mk(c.x / nsq, c.y / nsq, c.z / nsq));
        if (r.depth) r.depth[o] = dd / nsq;
    }
}

int32_t check_bvh(const ffsrl_bvh* b) {
    if (!b || b->num_envs <= 0 || !b->env_topology || !b->env_node_offset || !b->env_face_offset ||
        !b->topo_node_offset || !b->topo_tri_offset || !b->topo_max_level || !b->left_node || !b->first_tri_id ||
        !b->tri_count || !b->level || !b->tri_id || !b->aabb_min || !b->aabb_max || b->total_env_nodes <= 0)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh: missing arrays or empty");
    if (!b->node_box != !b->tri_pos)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh: node_box and tri_pos go together");
    if ((((uintptr_t)b->node_box) & 15) || (((uintptr_t)b->tri_pos) & 15))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh: node_box and tri_pos must be 16-byte aligned");
    return FFSRL_OK;
}

int32_t check_render(const ffsrl_render* r) {
    if (!r || r->num_envs <= 0 || r->resolution <= 0 || !r->vis_point || !r->vis_face || !r->vis_point_color ||
        !r->vertex_normal || !r->camera_pos || !r->camera_rot || r->num_cameras <= 0 ||
        (r->num_lights > 0 && (!r->light_dir || !r->light_intensity)) || !r->error_flag)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render: missing arrays");
    if (r->render_mode < 0 || r->render_mode > 4)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render: render_mode must be 0..4");
    if (r->env_objects && (!r->object_texture || !r->texture || !r->tex_coords || !r->tex_indices))
        return fail(FFSRL_ERR_INVALID_ARGUMENT,
                    "ffsrl_render: env_objects needs object_texture, texture, tex_coords and tex_indices");
    if (r->num_cameras != 1 && r->num_cameras != r->num_envs)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render: num_cameras must be 1 or num_envs");
    if (((uintptr_t)r->camera_rot) & 15)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render: camera_rot must be 16-byte aligned");
    return FFSRL_OK;
}

}  // namespace
}  // namespace ffsrl

using namespace ffsrl;

extern "C" int32_t ffsrl_bvh_refit_levels(const ffsrl_bvh* b, const float* pts, const int32_t* faces, void* stream) {
    if (int32_t st = check_bvh(b)) return st;
    if (!pts || !faces) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh_refit_levels: null points/faces");
    for (int L = b->max_level; L >= 0; --L)
        k_refit_level<<<grid_for(b->total_env_nodes, 256), 256, 0, (cudaStream_t)stream>>>(*b, pts, faces, L);
    FFSRL_LAUNCH_CHECK("ffsrl_bvh_refit_levels");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_bvh_refit_fused(const ffsrl_bvh* b, const float* pts, const int32_t* faces, void* stream) {
    if (int32_t st = check_bvh(b)) return st;
    if (!pts || !faces || !b->level_node || !b->level_start || !b->topo_level_offset)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh_refit_fused: needs level grouping arrays");
    k_refit_fused<<<b->num_envs, 256, 0, (cudaStream_t)stream>>>(*b, pts, faces, nullptr);
    FFSRL_LAUNCH_CHECK("ffsrl_bvh_refit_fused");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_render_reference(const ffsrl_render* r, const ffsrl_bvh* b, void* stream) {
    if (int32_t st = check_render(r)) return st;
    if (int32_t st = check_bvh(b)) return st;
    if (!r->normal_sum || !r->rays || !r->ray_depth)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render_reference: needs normal_sum, rays, ray_depth scratch");
    cudaStream_t s = (cudaStream_t)stream;
    const int P = r->num_vis_points, Fv = r->num_vis_faces;
    k_zero3<<<grid_for(P, 256), 256, 0, s>>>(r->normal_sum, P);
    if (Fv > 0) k_normal_sum<<<grid_for(Fv, 256), 256, 0, s>>>(r->vis_point, r->vis_face, r->normal_sum, Fv);
    k_normalize<<<grid_for(P, 256), 256, 0, s>>>(r->normal_sum, r->vertex_normal, P);
    long long rays = 4ll * r->resolution * r->resolution * r->num_envs;
    k_draw<<<grid_for(rays, 128), 128, 0, s>>>(*r, *b);
    long long pix = (long long)r->resolution * r->resolution * r->num_envs;
    k_downsample<<<grid_for(pix, 256), 256, 0, s>>>(*r);
    FFSRL_LAUNCH_CHECK("ffsrl_render_reference");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_render_fused(const ffsrl_render* r, const ffsrl_bvh* b, void* stream) {
    if (int32_t st = check_render(r)) return st;
    if (int32_t st = check_bvh(b)) return st;
    if (!r->point_face_start || !r->point_face)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render_fused: needs the point->face CSR");
    cudaStream_t s = (cudaStream_t)stream;
    const int P = r->num_vis_points;
    k_normal_gather<<<grid_for(P, 256), 256, 0, s>>>(r->vis_point, r->vis_face, r->point_face_start, r->point_face,
                                                     r->vertex_normal, P);
    const int tiles = ((r->resolution + 7) / 8) * ((r->resolution + 7) / 8);
    k_rays<<<(unsigned)((long long)tiles * r->num_envs), 256, 0, s>>>(*r, *b, nullptr, 0);
    FFSRL_LAUNCH_CHECK("ffsrl_render_fused");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_bvh_refit_fused_envs(const ffsrl_bvh* b, const float* pts, const int32_t* faces,
                                              const int32_t* env_ids, int32_t n, void* stream) {
    if (int32_t st = check_bvh(b)) return st;
    if (n < 0 || (n > 0 && (!pts || !faces || !env_ids || !b->level_node || !b->level_start || !b->topo_level_offset)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh_refit_fused_envs");
    if (n == 0) return FFSRL_OK;
    k_refit_fused<<<n, 256, 0, (cudaStream_t)stream>>>(*b, pts, faces, env_ids);
    FFSRL_LAUNCH_CHECK("ffsrl_bvh_refit_fused_envs");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_render_fused_envs(const ffsrl_render* r, const ffsrl_bvh* b, const int32_t* env_ids,
                                           int32_t n, void* stream) {
    if (int32_t st = check_render(r)) return st;
    if (int32_t st = check_bvh(b)) return st;
    if (n < 0 || (n > 0 && (!env_ids || !r->point_face_start || !r->point_face || !r->env_point_start)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render_fused_envs: needs env ids, point->face CSR, env point ranges");
    if (n == 0) return FFSRL_OK;
    cudaStream_t s = (cudaStream_t)stream;
    k_normal_gather_envs<<<n, 256, 0, s>>>(r->vis_point, r->vis_face, r->point_face_start, r->point_face,
                                           r->vertex_normal, r->env_point_start, env_ids, r->num_envs);
    const int tiles = ((r->resolution + 7) / 8) * ((r->resolution + 7) / 8);
    k_rays<<<(unsigned)((long long)tiles * n), 256, 0, s>>>(*r, *b, env_ids, n);
    FFSRL_LAUNCH_CHECK("ffsrl_render_fused_envs");
    return FFSRL_OK;
}
