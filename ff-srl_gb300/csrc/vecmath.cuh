// vecmath.cuh -- device vec3 arithmetic with the reference's (Warp 0.10.1) semantics.
//
// Expressions are written in the reference's association order.  Built-ins follow
// their mathematics: length = sqrt(dot), dot = (x*x' + y*y') + z*z',
// normalize(v) = v/|v| for |v| > 0 else 0, min/max = a<b?a:b / a>b?a:b.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ffsrl {

// FLOAT_EPSILON = sys.float_info.epsilon (integrator.py:8), compared in float32
#define FFSRL_FLOAT_EPS 2.220446049250313e-16f

struct v3 { float x, y, z; };
__device__ __forceinline__ v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ v3 operator+(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 operator-(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 operator-(v3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ v3 operator*(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ v3 operator*(float s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ v3 operator/(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(v3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ v3 normalize(v3 a) {
    float l = length(a);
    if (l > 0.0f) return a / l;
    return mk(0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ float fmin_ref(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float fmax_ref(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ v3 vmin(v3 a, v3 b) { return mk(fmin_ref(a.x, b.x), fmin_ref(a.y, b.y), fmin_ref(a.z, b.z)); }
__device__ __forceinline__ v3 vmax(v3 a, v3 b) { return mk(fmax_ref(a.x, b.x), fmax_ref(a.y, b.y), fmax_ref(a.z, b.z)); }

__device__ __forceinline__ v3 ld3(const float* __restrict__ p, long long i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void st3(float* __restrict__ p, long long i, v3 v) {
    p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z;
}
__device__ __forceinline__ void atomic_add3(float* p, long long i, v3 v) {
    atomicAdd(p + 3 * i, v.x); atomicAdd(p + 3 * i + 1, v.y); atomicAdd(p + 3 * i + 2, v.z);
}

// The same three float additions in two atomic instructions: the 8-byte-aligned pair of
// the entry (x, y for an even i, y, z for an odd one) as one float2 atomic (global memory,
// sm_90 and later), the other component alone.  Each component is still added by one
// float atomic, so the sums are those of atomic_add3 in some order.  Falls back to
// atomic_add3 when p is not 8-byte aligned.
__device__ __forceinline__ void atomic_add3_pair(float* p, long long i, v3 v) {
    if (reinterpret_cast<uintptr_t>(p) & 7) {
        atomic_add3(p, i, v);
    } else if ((i & 1) == 0) {
        atomicAdd(reinterpret_cast<float2*>(p + 3 * i), make_float2(v.x, v.y));
        atomicAdd(p + 3 * i + 2, v.z);
    } else {
        atomicAdd(p + 3 * i, v.x);
        atomicAdd(reinterpret_cast<float2*>(p + 3 * i + 1), make_float2(v.y, v.z));
    }
}

// closestPointOnEdge (integrator.py:1520-1534)
__device__ __forceinline__ v3 closest_on_edge(v3 p, v3 a, v3 b) {
    v3 d = b - a;
    float t;
    if (length(d) < FFSRL_FLOAT_EPS) {
        t = 0.5f;
    } else {
        float ld = length(d);
        float d2 = ld * ld;
        t = dot(d, p - a) / d2;
        if (t < 0.0f) t = 0.0f;
        else if (t > 1.0f) t = 1.0f;
    }
    return a + d * t;
}

// triangle_closest_point_barycentric (integrator.py:1536-1581)
__device__ __forceinline__ v3 closest_bary(v3 a, v3 b, v3 c, v3 p) {
    v3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return mk(1.0f, 0.0f, 0.0f);
    v3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return mk(0.0f, 1.0f, 0.0f);
    float vc = d1 * d4 - d3 * d2;
    float v = d1 / (d1 - d3);
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return mk(1.0f - v, v, 0.0f);
    v3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return mk(0.0f, 0.0f, 1.0f);
    float vb = d5 * d2 - d1 * d6;
    float w = d2 / (d2 - d6);
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return mk(1.0f - w, 0.0f, w);
    float va = d3 * d6 - d5 * d4;
    w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) return mk(0.0f, w, 1.0f - w);
    float denom = 1.0f / (va + vb + vc);
    v = vb * denom;
    w = vc * denom;
    return mk(1.0f - v - w, v, w);
}

// checkSdfCapsuleCollision (integrator.py:1302-1355).  Note the reference passes the
// barycentric triple of the line/plane point (not the point) to closestPointOnEdge.
__device__ __forceinline__ bool capsule_response(v3 tip, v3 base, float radius, v3 n, v3 centre, v3 pA, v3 pB,
                                                 v3 pC, float ks, v3& rA, v3& rB, v3& rC) {
    v3 cn = normalize(tip - base);
    v3 off = cn * radius;
    v3 posA = base + off;
    v3 posB = tip - off;
    float denom = dot(n, cn);
    if (fabsf(denom) < FFSRL_FLOAT_EPS) return false;
    float t = dot(n, centre - base) / denom;
    v3 lp = base + cn * t;
    v3 ref = closest_bary(pA, pB, pC, lp);
    v3 sc = closest_on_edge(ref, posA, posB);
    v3 bary = closest_bary(pA, pB, pC, sc);
    v3 contact = pA * bary.x + pB * bary.y + pC * bary.z;
    v3 sv = sc - contact;
    float dist = length(sv);
    float pen = radius / length(sv) - 1.0f;
    v3 pv = mk(pen * sv.x, pen * sv.y, pen * sv.z);
    float plen = length(pv);
    v3 pn = normalize(pv);
    float sq = bary.x * bary.x + bary.y * bary.y + bary.z * bary.z;
    if (sq < FFSRL_FLOAT_EPS) return false;
    v3 resp = pn * (plen / sq) * ks;
    if (dist > radius) return false;
    rA = resp * bary.x; rB = resp * bary.y; rC = resp * bary.z;
    return true;
}

}  // namespace ffsrl
