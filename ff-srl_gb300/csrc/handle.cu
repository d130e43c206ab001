// handle.cu -- an owning handle over the batched step for C callers: the library uploads a
// model given in host memory (the arrays of SimModelDO, modelDO.py:1141-1246), builds its
// batched plan, steps it, and hands out the device pointers so the caller can read and
// write state, tool and grasp arrays in place between steps.
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "ffsrl_internal.h"

using namespace ffsrl;

struct ffsrl_handle {
    ffsrl_model dev{};
    ffsrl_params params{};
    ffsrl_batch* plan = nullptr;
    std::vector<void*> owned;
};

namespace {

// device copy of `count` elements of a host array (zero-filled when the host array is
// NULL and `always` is set; left NULL otherwise)
template <class T>
int32_t upload(ffsrl_handle* h, T** dst, const T* src, int64_t count, bool always) {
    *dst = nullptr;
    if (count <= 0 || (!src && !always)) return FFSRL_OK;
    void* p = nullptr;
    FFSRL_CUDA_TRY(cudaMalloc(&p, sizeof(T) * (size_t)count));
    h->owned.push_back(p);
    if (src) FFSRL_CUDA_TRY(cudaMemcpy(p, src, sizeof(T) * (size_t)count, cudaMemcpyHostToDevice));
    else FFSRL_CUDA_TRY(cudaMemset(p, 0, sizeof(T) * (size_t)count));
    *dst = static_cast<T*>(p);
    return FFSRL_OK;
}

template <class T>
int32_t upload_c(ffsrl_handle* h, const T** dst, const T* src, int64_t count, bool always) {
    T* p = nullptr;
    int32_t r = upload(h, &p, src, count, always);
    *dst = p;
    return r;
}

void release(ffsrl_handle* h) {
    if (h->plan) ffsrl_batch_destroy(h->plan);
    for (void* p : h->owned) cudaFree(p);
    delete h;
}

}  // namespace

extern "C" int32_t ffsrl_create(const ffsrl_model* m, const ffsrl_params* p, int32_t block_threads,
                                ffsrl_handle** out) {
    if (!out) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_create: out is NULL");
    *out = nullptr;
    if (!m || !p || m->num_envs <= 0 || m->num_vertices <= 0 || !m->vertex || !m->inverse_mass ||
        !m->env_vertex_start || !m->env_tet_start || !m->env_edge_start || !m->env_tri_start || !m->laparoscope_base ||
        !m->laparoscope_tip || !m->laparoscope_radius || block_threads < 0)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_create: missing host arrays or sizes");
    const int64_t V = m->num_vertices, T = m->num_tetrahedrons, E = m->num_edges, F = m->num_triangles;
    const int64_t N = m->num_envs, Cn = m->num_connectors;
    auto* h = new ffsrl_handle;
    ffsrl_model& d = h->dev;
    d.num_vertices = m->num_vertices; d.num_tetrahedrons = m->num_tetrahedrons; d.num_edges = m->num_edges;
    d.num_triangles = m->num_triangles; d.num_connectors = m->num_connectors; d.num_envs = m->num_envs;
    int32_t st = FFSRL_OK;
    auto chk = [&](int32_t r) { if (r && !st) st = r; };
    chk(upload(h, &d.vertex, m->vertex, 3 * V, true));
    chk(upload(h, &d.predicted_vertex, m->predicted_vertex, 3 * V, true));
    chk(upload(h, &d.velocity, m->velocity, 3 * V, true));
    chk(upload(h, &d.dp, m->dp, 3 * V, true));
    chk(upload(h, &d.constraints_number, m->constraints_number, V, true));
    chk(upload(h, &d.collision_dp, m->collision_dp, 3 * V, true));
    chk(upload_c(h, &d.inverse_mass, m->inverse_mass, V, true));
    chk(upload_c(h, &d.tetrahedron, m->tetrahedron, 4 * T, false));
    chk(upload_c(h, &d.tetrahedron_rest_volume, m->tetrahedron_rest_volume, T, false));
    chk(upload_c(h, &d.active_tetrahedron, m->active_tetrahedron, T, false));
    chk(upload_c(h, &d.tetrahedron_dm_inv, m->tetrahedron_dm_inv, 9 * T, false));
    chk(upload(h, &d.tetrahedron_lambda, m->tetrahedron_lambda, T, true));
    chk(upload_c(h, &d.xpbd_rest_volume, m->xpbd_rest_volume, T, false));
    chk(upload_c(h, &d.edge, m->edge, 2 * E, false));
    chk(upload_c(h, &d.edge_rest_length, m->edge_rest_length, E, false));
    chk(upload_c(h, &d.active_edge, m->active_edge, E, false));
    chk(upload(h, &d.edge_lambda, m->edge_lambda, E, true));
    chk(upload_c(h, &d.triangle, m->triangle, 3 * F, false));
    chk(upload_c(h, &d.tri_to_env, m->tri_to_env, F, false));
    chk(upload_c(h, &d.hole, m->hole, F, true));
    chk(upload_c(h, &d.vertex_to_env, m->vertex_to_env, V, false));
    chk(upload_c(h, &d.active_drag_constraint, m->active_drag_constraint, V, true));
    chk(upload_c(h, &d.laparoscope_base, m->laparoscope_base, 12 * N, true));
    chk(upload_c(h, &d.laparoscope_tip, m->laparoscope_tip, 12 * N, true));
    chk(upload_c(h, &d.laparoscope_radius, m->laparoscope_radius, 4 * N, true));
    chk(upload(h, &d.laparoscope_in_collision, m->laparoscope_in_collision, N, true));
    chk(upload_c(h, &d.connector_triangle_id, m->connector_triangle_id, 3 * Cn, false));
    chk(upload_c(h, &d.connector_tri_bar, m->connector_tri_bar, 3 * Cn, false));
    chk(upload_c(h, &d.connector_vertex_id, m->connector_vertex_id, Cn, false));
    chk(upload_c(h, &d.connector_rest_dist, m->connector_rest_dist, Cn, false));
    chk(upload_c(h, &d.env_vertex_start, m->env_vertex_start, N + 1, true));
    chk(upload_c(h, &d.env_tet_start, m->env_tet_start, N + 1, true));
    chk(upload_c(h, &d.env_edge_start, m->env_edge_start, N + 1, true));
    chk(upload_c(h, &d.env_tri_start, m->env_tri_start, N + 1, true));
    if (st) {
        std::string msg = std::string("ffsrl_create: upload: ") + ffsrl_last_error();
        release(h);
        return fail(st, msg);
    }
    h->params = *p;
    ffsrl_batch_options o{};
    o.block_threads = block_threads;
    o.deterministic = 1;
    if ((st = ffsrl_batch_create(m, &h->dev, &h->params, &o, &h->plan))) {
        std::string msg = ffsrl_last_error();
        h->plan = nullptr;
        release(h);
        return fail(st, msg);
    }
    *out = h;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_destroy(ffsrl_handle* h) {
    if (!h) return FFSRL_OK;
    cudaDeviceSynchronize();
    release(h);
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_step(ffsrl_handle* h, int32_t n_steps, void* stream) {
    if (!h) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_step: handle is NULL");
    return ffsrl_batch_step(h->plan, n_steps, stream);
}

extern "C" int32_t ffsrl_get_device_model(const ffsrl_handle* h, ffsrl_model* out, ffsrl_batch** plan) {
    if (!h || !out) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_get_device_model");
    *out = h->dev;
    if (plan) *plan = h->plan;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_set_tool(ffsrl_handle* h, const float* base, const float* tip, const float* radius,
                                  int32_t from_host, void* stream) {
    if (!h) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_set_tool: handle is NULL");
    const size_t n = (size_t)h->dev.num_envs;
    const cudaMemcpyKind k = from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    cudaStream_t s = (cudaStream_t)stream;
    if (base) FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)h->dev.laparoscope_base, base, 48 * n, k, s));
    if (tip) FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)h->dev.laparoscope_tip, tip, 48 * n, k, s));
    if (radius) FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)h->dev.laparoscope_radius, radius, 16 * n, k, s));
    if (from_host) FFSRL_CUDA_TRY(cudaStreamSynchronize(s));  // the host arrays may go after the call
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_set_drag(ffsrl_handle* h, const float* drag, int32_t from_host, void* stream) {
    if (!h || !drag) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_set_drag");
    cudaStream_t s = (cudaStream_t)stream;
    FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)h->dev.active_drag_constraint, drag, 4 * (size_t)h->dev.num_vertices,
                                   from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    if (from_host) FFSRL_CUDA_TRY(cudaStreamSynchronize(s));
    return FFSRL_OK;
}
