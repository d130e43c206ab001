// cutting.cu -- tissue cutting and heating kernels of the reference
// (FF_SRL/FF_SRL/integrator.py:700-918, 1153-1185, 1406-1518, 1583-1605): edge and tet
// breakers that accumulate overstretch, the checks that flip broken elements and open
// holes in the surface, heat conduction between neighbouring tets, the instrument's heat
// source, the cut of edges that cross the clamp triangle, and the fade of flipped
// elements' active values.  The reference's DO step does not launch them (its legacy
// integrator has the launches commented out, integrator.py:2182-2230); they are library
// calls here, over the env-major arrays of many envs.
//
// One thread per element, as the reference.  Where the reference's result depends on
// which thread writes last (a vertex's heat, written by every tet that holds it), the
// tet with the highest id wins, as in a serial run in thread order.  The reference's
// single-instrument calls (capsule tips 1 and 2, the clamp triangle of tips 0..2) take
// the element's env's instrument here (tips 4e+k); with no env map, env 0's, which is
// the reference.  A tet scan for an edge covers the edge's env only: tets of other envs
// share no vertex with it, so the outcome is the reference's full scan.  Index quirks of
// the reference are kept and guarded: the breaker check flips flipTetrahedron[edge id]
// (integrator.py:772-774) only where that id is a tet id, and a map entry of -1 opens no
// hole.  Built without FMA contraction, like the CPU restatement.
#include <cuda_runtime.h>
#include <cstdint>
#include "ffsrl_internal.h"
#include "vecmath.cuh"

namespace ffsrl {
namespace {

__device__ __forceinline__ bool holds(const int* q, int v) { return v == q[0] || v == q[1] || v == q[2] || v == q[3]; }

// tets [t0, t1) to scan for edge k (all tets without an env table)
__device__ __forceinline__ void tet_range(const int* env_of, const int* env_tet_start, int nt, int k, int& t0,
                                          int& t1) {
    t0 = 0;
    t1 = nt;
    if (env_of && env_tet_start) {
        const int e = env_of[k];
        t0 = env_tet_start[e];
        t1 = env_tet_start[e + 1];
    }
}

// edgeBreakerKernel (integrator.py:700-731)
__global__ void k_edge_breaker(const float* __restrict__ xp, const int* __restrict__ edge,
                               const float* __restrict__ rest, const float* __restrict__ active, float* value,
                               float factor, float threshold, int ne) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne || active[t] == 0.0f) return;
    const float L0 = rest[t];
    if (L0 < FFSRL_FLOAT_EPS) return;
    const float len = length(ld3(xp, edge[2 * t + 1]) - ld3(xp, edge[2 * t]));
    if (len < FFSRL_FLOAT_EPS) return;
    const float C = len / L0 - 1.0f;
    if (C > threshold) value[t] = value[t] + (C - threshold) * factor;
}

// checkEdgeBreakerKernel (integrator.py:733-775)
__global__ void k_check_edge_breaker(const float* __restrict__ value, const int* __restrict__ edge,
                                     const float* __restrict__ active_edge, int* flip_edges,
                                     const int* __restrict__ tet, int nt, const float* __restrict__ active_tet,
                                     int* flip_tets, const int* __restrict__ edge_tris, int* holes, float limit,
                                     const int* __restrict__ edge_env, const int* __restrict__ env_tet_start, int ne) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne || !(value[t] > limit)) return;
    if (flip_edges[t] == 0 && active_edge[t] == 1.0f) flip_edges[t] = -1;
    const int a = edge[2 * t], b = edge[2 * t + 1];
    const int ta = edge_tris[2 * t], tb = edge_tris[2 * t + 1];
    if (ta > -1) holes[ta] = 1;
    if (tb > -1) holes[tb] = 1;
    if (t >= nt || flip_tets[t] != 0 || !(active_tet[t] == 1.0f)) return;  // nothing the scan could change
    int t0, t1;
    tet_range(edge_env, env_tet_start, nt, t, t0, t1);
    for (int i = t0; i < t1; ++i) {
        const int* q = tet + 4 * i;
        if (holds(q, a) && holds(q, b)) {
            flip_tets[t] = -1;  // the reference's tet flag indexed by the edge id
            return;
        }
    }
}

// tetrahedronBreaker (integrator.py:777-818): signed volume beyond the rest volume
__global__ void k_tet_breaker(const float* __restrict__ xp, const int* __restrict__ tet,
                              const float* __restrict__ rest, const float* __restrict__ active, float* value,
                              float factor, int nt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt || !(active[t] == 1.0f)) return;
    const v3 pa = ld3(xp, tet[4 * t]);
    const v3 p1 = ld3(xp, tet[4 * t + 1]) - pa, p2 = ld3(xp, tet[4 * t + 2]) - pa, p3 = ld3(xp, tet[4 * t + 3]) - pa;
    const float C = dot(cross(p1, p2), p3) / 6.0f - rest[t];
    if (C > 0.0f) value[t] = value[t] + C * factor;
}

// tetrahedronHeatPropagation (integrator.py:820-847)
__global__ void k_heat_propagation(const float* __restrict__ active, const int* __restrict__ nbr,
                                   const float* __restrict__ heat, float* new_heat, float conduction, float transfer,
                                   float loss, int nt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt || active[t] == 0.0f) return;
    const float h = heat[t];
    float avg = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const int n = nbr[4 * t + i];
        if (n > -1 && active[n] > 0.0f) avg = avg + (heat[n] - h) * conduction;
    }
    new_heat[t] = h * (1.0f - loss) + avg * transfer;
}

// tetrahedronHeatUpdate (integrator.py:849-872), first pass: the highest tet id holding
// each vertex among the active tets
__global__ void k_heat_owner(const float* __restrict__ active, const int* __restrict__ tet, int* owner, int nt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt || !(active[t] > 0.0f)) return;
    for (int k = 0; k < 4; ++k) atomicMax(owner + tet[4 * t + k], t);
}

// second pass: tet heat from the propagation, vertex heat from its owning tet
__global__ void k_heat_update(float* heat, const float* __restrict__ new_heat, const float* __restrict__ active,
                              const int* __restrict__ tet, const int* __restrict__ owner, float* vertex_heat, int nt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    if (active[t] > 0.0f) {
        const float h = new_heat[t];
        heat[t] = h;
        for (int k = 0; k < 4; ++k) {
            const int v = tet[4 * t + k];
            if (owner[v] == t) vertex_heat[v] = h / 4.0f;
        }
    } else {
        heat[t] = 0.0f;
    }
}

// checkTetrahedronHeat (integrator.py:874-895) and, with rest volumes,
// checkTetrahedronHeatVolumeProportional (integrator.py:897-918)
__global__ void k_check_heat(const float* __restrict__ heat, int* flip, const float* __restrict__ rest,
                             const int* __restrict__ tet_tris, int* holes, float limit, int nt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const float h = heat[t];
    if (rest ? !(h > limit * rest[t]) : !(h > limit)) return;
    if (rest || flip[t] == 0) {
        flip[t] = -1;
        for (int i = 0; i < 4; ++i) {
            const int f = tet_tris[4 * t + i];
            if (f > -1) holes[f] = 1;
        }
    }
}

// heatLaparoscope (integrator.py:1153-1185): surface triangles within the sphere between
// the clamp tips heat their tet.  The increments are equal, so their sum does not depend
// on the order of the adds.
__global__ void k_heat_laparoscope(const int* __restrict__ tri, const float* __restrict__ pos,
                                   const float* __restrict__ active, float* heat, const int* __restrict__ tri_tet,
                                   const float* __restrict__ tips, const int* __restrict__ tri_env, float radius,
                                   float quantum, int nf) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf) return;
    const int e = tri_env ? tri_env[t] : 0;
    const v3 centre = (ld3(tips, 4 * e + 1) + ld3(tips, 4 * e + 2)) / 2.0f;
    const v3 a = ld3(pos, tri[3 * t]), b = ld3(pos, tri[3 * t + 1]), c = ld3(pos, tri[3 * t + 2]);
    const v3 bary = closest_bary(a, b, c, centre);
    const v3 closest = a * bary.x + b * bary.y + c * bary.z;
    if (length(closest - centre) < radius) {
        const int k = tri_tet[t];
        if (k > -1 && active[k] > 0.0f) atomicAdd(heat + k, quantum);
    }
}

// checkSegmentTriangleIntersection (integrator.py:1471-1518): 1 when segment sA-sB
// crosses triangle pA pB pC, 2 when it lies in the triangle's plane, 0 otherwise, -1 for
// a degenerate triangle
__device__ int segment_triangle(v3 pA, v3 pB, v3 pC, v3 sA, v3 sB) {
    const v3 u = pB - pA, v = pC - pA;
    const v3 n = cross(u, v);
    if (n.x == 0.0f && n.y == 0.0f && n.z == 0.0f) return -1;
    const v3 dir = sB - sA, w0 = sA - pA;
    const float a = -dot(n, w0), b = dot(n, dir);
    if (fabsf(b) < FFSRL_FLOAT_EPS) return a == 0.0f ? 2 : 0;
    const float r = a / b;
    if (r < 0.0f || r > 1.0f) return 0;
    const v3 I = sA + r * dir;
    const float uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
    const v3 w = I - pA;
    const float wu = dot(w, u), wv = dot(w, v);
    const float D = uv * uv - uu * vv;
    const float s = (uv * wv - vv * wu) / D;
    if (s < 0.0f || s > 1.0f) return 0;
    const float tt = (uv * wu - uu * wv) / D;
    if (tt < 0.0f || (s + tt) > 1.0f) return 0;
    return 1;
}

// findIntersectingEdges (integrator.py:1406-1458): an edge crossing the triangle of the
// rod tip and the right and left clamp tips is flipped, opens its surface triangles and
// flips every active tet holding it
__global__ void k_cut_edges(const float* __restrict__ pos, const float* __restrict__ tips,
                            const int* __restrict__ edge, const float* __restrict__ active_edge, int* flip_edges,
                            const int* __restrict__ tet, int nt, const float* __restrict__ active_tet, int* flip_tets,
                            const int* __restrict__ edge_tris, int* holes, const int* __restrict__ edge_env,
                            const int* __restrict__ env_tet_start, int ne) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne) return;
    const int e = edge_env ? edge_env[t] : 0;
    const int a = edge[2 * t], b = edge[2 * t + 1];
    if (segment_triangle(ld3(tips, 4 * e), ld3(tips, 4 * e + 2), ld3(tips, 4 * e + 1), ld3(pos, a), ld3(pos, b)) != 1)
        return;
    if (flip_edges[t] == 0 && active_edge[t] == 1.0f) flip_edges[t] = -1;
    const int ta = edge_tris[2 * t], tb = edge_tris[2 * t + 1];
    if (ta > -1) holes[ta] = 1;
    if (tb > -1) holes[tb] = 1;
    int t0, t1;
    tet_range(edge_env, env_tet_start, nt, t, t0, t1);
    for (int i = t0; i < t1; ++i) {
        const int* q = tet + 4 * i;
        // other threads only ever write -1 here, so a stale 0 read sets the same value
        if (holds(q, a) && holds(q, b) && flip_tets[i] == 0 && active_tet[i] == 1.0f) flip_tets[i] = -1;
    }
}

// inDeCreaseActiveValues (integrator.py:1583-1605): a flipped element's active value
// steps along the table sqrt(k / steps), up for flip > 0 and down for flip < 0; the flip
// counter returns to 0 after `steps` steps.  Counters beyond the table are left alone.
__global__ void k_fade_active(int* flip, float* active, const float* __restrict__ table, int steps, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int f = flip[t];
    if (f == 0 || f > steps || f < -steps) return;
    int k;
    if (f > 0) {
        k = f;
        flip[t] = f + 1;
    } else {
        k = steps + f;
        flip[t] = f - 1;
    }
    active[t] = table[k];
    if (abs(f) >= steps) flip[t] = 0;
}

inline unsigned blocks(int n) { return grid_for(n, 256); }

}  // namespace
}  // namespace ffsrl

using namespace ffsrl;

extern "C" int32_t ffsrl_edge_breaker(const float* predicted, const int32_t* edge, const float* rest_length,
                                      const float* active_edge, float* breaker_value, int32_t num_edges,
                                      float break_factor, float break_threshold, void* stream) {
    if (num_edges < 0 || (num_edges > 0 && (!predicted || !edge || !rest_length || !active_edge || !breaker_value)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_edge_breaker");
    if (!num_edges) return FFSRL_OK;
    k_edge_breaker<<<blocks(num_edges), 256, 0, (cudaStream_t)stream>>>(predicted, edge, rest_length, active_edge,
                                                                         breaker_value, break_factor, break_threshold,
                                                                         num_edges);
    FFSRL_LAUNCH_CHECK("ffsrl_edge_breaker");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_check_edge_breaker(const float* breaker_value, const int32_t* edge, const float* active_edge,
                                            int32_t* flip_edges, int32_t num_edges, const int32_t* tetrahedron,
                                            int32_t num_tets, const float* active_tet, int32_t* flip_tets,
                                            const int32_t* edge_to_triangles, int32_t* holes, float break_limit,
                                            const int32_t* edge_to_env, const int32_t* env_tet_start, void* stream) {
    if (num_edges < 0 || num_tets < 0 ||
        (num_edges > 0 && (!breaker_value || !edge || !active_edge || !flip_edges || !edge_to_triangles || !holes)) ||
        (num_tets > 0 && (!tetrahedron || !active_tet || !flip_tets)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_check_edge_breaker");
    if (!num_edges) return FFSRL_OK;
    k_check_edge_breaker<<<blocks(num_edges), 256, 0, (cudaStream_t)stream>>>(
        breaker_value, edge, active_edge, flip_edges, tetrahedron, num_tets, active_tet, flip_tets, edge_to_triangles,
        holes, break_limit, edge_to_env, env_tet_start, num_edges);
    FFSRL_LAUNCH_CHECK("ffsrl_check_edge_breaker");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_tetrahedron_breaker(const float* predicted, const int32_t* tetrahedron,
                                             const float* rest_volume, const float* active_tet, float* breaker_value,
                                             int32_t num_tets, float break_factor, void* stream) {
    if (num_tets < 0 || (num_tets > 0 && (!predicted || !tetrahedron || !rest_volume || !active_tet || !breaker_value)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_tetrahedron_breaker");
    if (!num_tets) return FFSRL_OK;
    k_tet_breaker<<<blocks(num_tets), 256, 0, (cudaStream_t)stream>>>(predicted, tetrahedron, rest_volume, active_tet,
                                                                       breaker_value, break_factor, num_tets);
    FFSRL_LAUNCH_CHECK("ffsrl_tetrahedron_breaker");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_heat_propagation(const float* active_tet, const int32_t* neighbors, const float* heat,
                                          float* new_heat, int32_t num_tets, float conduction, float transfer,
                                          float loss, void* stream) {
    if (num_tets < 0 || (num_tets > 0 && (!active_tet || !neighbors || !heat || !new_heat)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_heat_propagation");
    if (!num_tets) return FFSRL_OK;
    k_heat_propagation<<<blocks(num_tets), 256, 0, (cudaStream_t)stream>>>(active_tet, neighbors, heat, new_heat,
                                                                            conduction, transfer, loss, num_tets);
    FFSRL_LAUNCH_CHECK("ffsrl_heat_propagation");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_heat_update(float* heat, const float* new_heat, const float* active_tet,
                                     const int32_t* tetrahedron, float* vertex_heat, int32_t* owner_scratch,
                                     int32_t num_tets, int32_t num_vertices, void* stream) {
    if (num_tets < 0 || num_vertices < 0 ||
        (num_tets > 0 && (!heat || !new_heat || !active_tet || !tetrahedron || !vertex_heat || !owner_scratch)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_heat_update");
    if (!num_tets) return FFSRL_OK;
    cudaStream_t s = (cudaStream_t)stream;
    FFSRL_CUDA_TRY(cudaMemsetAsync(owner_scratch, 0xff, sizeof(int32_t) * (size_t)num_vertices, s));
    k_heat_owner<<<blocks(num_tets), 256, 0, s>>>(active_tet, tetrahedron, owner_scratch, num_tets);
    k_heat_update<<<blocks(num_tets), 256, 0, s>>>(heat, new_heat, active_tet, tetrahedron, owner_scratch, vertex_heat,
                                                   num_tets);
    FFSRL_LAUNCH_CHECK("ffsrl_heat_update");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_check_heat(const float* heat, int32_t* flip_tets, const float* rest_volume,
                                    const int32_t* tet_to_triangles, int32_t* holes, float heat_limit,
                                    int32_t num_tets, void* stream) {
    if (num_tets < 0 || (num_tets > 0 && (!heat || !flip_tets || !tet_to_triangles || !holes)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_check_heat");
    if (!num_tets) return FFSRL_OK;
    k_check_heat<<<blocks(num_tets), 256, 0, (cudaStream_t)stream>>>(heat, flip_tets, rest_volume, tet_to_triangles,
                                                                      holes, heat_limit, num_tets);
    FFSRL_LAUNCH_CHECK("ffsrl_check_heat");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_heat_laparoscope(const int32_t* triangle, const float* positions, const float* active_tet,
                                          float* heat, const int32_t* triangle_to_tet, const float* capsule_tips,
                                          const int32_t* triangle_to_env, float sphere_radius, float heat_quantum,
                                          int32_t num_triangles, void* stream) {
    if (num_triangles < 0 ||
        (num_triangles > 0 && (!triangle || !positions || !active_tet || !heat || !triangle_to_tet || !capsule_tips)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_heat_laparoscope");
    if (!num_triangles) return FFSRL_OK;
    k_heat_laparoscope<<<blocks(num_triangles), 256, 0, (cudaStream_t)stream>>>(
        triangle, positions, active_tet, heat, triangle_to_tet, capsule_tips, triangle_to_env, sphere_radius,
        heat_quantum, num_triangles);
    FFSRL_LAUNCH_CHECK("ffsrl_heat_laparoscope");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_cut_edges(const float* positions, const float* capsule_tips, const int32_t* edge,
                                   const float* active_edge, int32_t* flip_edges, int32_t num_edges,
                                   const int32_t* tetrahedron, int32_t num_tets, const float* active_tet,
                                   int32_t* flip_tets, const int32_t* edge_to_triangles, int32_t* holes,
                                   const int32_t* edge_to_env, const int32_t* env_tet_start, void* stream) {
    if (num_edges < 0 || num_tets < 0 ||
        (num_edges > 0 &&
         (!positions || !capsule_tips || !edge || !active_edge || !flip_edges || !edge_to_triangles || !holes)) ||
        (num_tets > 0 && (!tetrahedron || !active_tet || !flip_tets)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_cut_edges");
    if (!num_edges) return FFSRL_OK;
    k_cut_edges<<<blocks(num_edges), 256, 0, (cudaStream_t)stream>>>(
        positions, capsule_tips, edge, active_edge, flip_edges, tetrahedron, num_tets, active_tet, flip_tets,
        edge_to_triangles, holes, edge_to_env, env_tet_start, num_edges);
    FFSRL_LAUNCH_CHECK("ffsrl_cut_edges");
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_update_active_values(int32_t* flip, float* active, const float* table, int32_t steps,
                                              int32_t n, void* stream) {
    if (n < 0 || steps < 1 || (n > 0 && (!flip || !active || !table)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_update_active_values");
    if (!n) return FFSRL_OK;
    k_fade_active<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(flip, active, table, steps, n);
    FFSRL_LAUNCH_CHECK("ffsrl_update_active_values");
    return FFSRL_OK;
}
