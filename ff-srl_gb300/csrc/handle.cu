// handle.cu -- an owning handle over the batched step for C callers: the library uploads a
// model given in host memory (the arrays of SimModelDO, modelDO.py:1141-1246), builds its
// batched plan, steps it, and hands out the device pointers so the caller can read and
// write state, tool and grasp arrays in place between steps.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <map>
#include <numeric>
#include <string>
#include <vector>
#include "ffsrl_internal.h"

using namespace ffsrl;

struct ffsrl_handle {
    ffsrl_model dev{};
    ffsrl_params params{};
    ffsrl_batch* plan = nullptr;
    std::vector<void*> owned;
    // observation (ffsrl_attach_render): visual mesh, per-topology BVHs, render buffers
    bool has_render = false;
    ffsrl_bvh bvh{};
    ffsrl_render render{};
    float* vis_point = nullptr;
    const int32_t* point_to_vertex = nullptr;
    int32_t num_map = 0;
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
    chk(upload(h, &d.vertex, m->vertex, 3 * V, true));  // first: the remap below reads it
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
    o.block_threads = block_threads;  // reference arithmetic, fixed-point sums
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

// ---- observation: BVH refit and ray-cast of the handle's envs ---------------------------
extern "C" int32_t ffsrl_attach_render(ffsrl_handle* h, const ffsrl_render_config* c) {
    if (!h || !c || h->has_render || c->num_points <= 0 || c->num_faces <= 0 || !c->points || !c->faces ||
        !c->colors || c->num_map < 0 || (c->num_map > 0 && !c->point_to_vertex) || !c->env_point_start ||
        !c->env_face_start || c->resolution <= 0 || c->num_lights < 0 ||
        (c->num_lights > 0 && (!c->light_dir || !c->light_intensity)) || c->render_mode < 0 || c->render_mode > 4 ||
        c->render_mode == 1)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_attach_render: missing arrays, bad sizes or mode");
    const int N = h->dev.num_envs;
    const int64_t P = c->num_points, Fv = c->num_faces;
    const size_t owned0 = h->owned.size();  // buffers this call allocates come after these
    if (c->env_point_start[0] != 0 || c->env_point_start[N] != P || c->env_face_start[0] != 0 ||
        c->env_face_start[N] != Fv)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_attach_render: env ranges do not cover the points and faces");
    for (int64_t k = 0; k < 3 * Fv; ++k)
        if (c->faces[k] < 0 || c->faces[k] >= P) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_attach_render: face index");
    for (int64_t k = 0; k < c->num_map; ++k)
        if (c->point_to_vertex[2 * k] < 0 || c->point_to_vertex[2 * k] >= P || c->point_to_vertex[2 * k + 1] < 0 ||
            c->point_to_vertex[2 * k + 1] >= h->dev.num_vertices)
            return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_attach_render: remap pair out of range");
    // one BVH topology per distinct topology id, built on its first env's points (the
    // reference's binned SAH with 8 bins, bvh.py:456-518)
    std::vector<int> env_topo(N);
    std::map<int, int> ids;
    std::vector<int> topo_env;
    for (int e = 0; e < N; ++e) {
        const int key = c->env_topology ? c->env_topology[e] : e;
        auto it = ids.find(key);
        if (it == ids.end()) { it = ids.emplace(key, (int)topo_env.size()).first; topo_env.push_back(e); }
        env_topo[e] = it->second;
        const int e0 = topo_env[it->second];
        if (c->env_face_start[e + 1] - c->env_face_start[e] != c->env_face_start[e0 + 1] - c->env_face_start[e0])
            return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_attach_render: envs of one topology differ in faces");
    }
    const int M = (int)topo_env.size();
    std::vector<int> left, first, count, level, tri, topo_node(M + 1, 0), topo_tri(M + 1, 0), topo_max(M);
    std::vector<int> level_node, level_start, topo_level(M + 1, 0);
    std::vector<std::vector<float>> tmin(M), tmax(M);
    for (int t = 0; t < M; ++t) {
        const int e = topo_env[t];
        const int p0 = c->env_point_start[e], np = c->env_point_start[e + 1] - p0;
        const int f0 = c->env_face_start[e], nf = c->env_face_start[e + 1] - f0;
        std::vector<int> lf(3 * (size_t)nf);
        for (int k = 0; k < 3 * nf; ++k) {
            lf[k] = c->faces[3ll * f0 + k] - p0;
            if (lf[k] < 0 || lf[k] >= np) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_attach_render: a face leaves its env");
        }
        const int cap = 2 * std::max(nf, 1);
        std::vector<int> L(cap), Fi(cap), Cn(cap), Lv(cap), Ti(std::max(nf, 1));
        std::vector<float> a0(3 * (size_t)cap), a1(3 * (size_t)cap);
        int nn = 0, ml = 0;
        if (int32_t r = ffsrl_bvh_build_host(c->points + 3ll * p0, lf.data(), np, nf, 8, L.data(), Fi.data(), Cn.data(),
                                             Lv.data(), Ti.data(), a0.data(), a1.data(), &nn, &ml))
            return r;
        left.insert(left.end(), L.begin(), L.begin() + nn);
        first.insert(first.end(), Fi.begin(), Fi.begin() + nn);
        count.insert(count.end(), Cn.begin(), Cn.begin() + nn);
        level.insert(level.end(), Lv.begin(), Lv.begin() + nn);
        tri.insert(tri.end(), Ti.begin(), Ti.begin() + nf);
        tmin[t].assign(a0.begin(), a0.begin() + 3 * (size_t)nn);
        tmax[t].assign(a1.begin(), a1.begin() + 3 * (size_t)nn);
        topo_node[t + 1] = topo_node[t] + nn;
        topo_tri[t + 1] = topo_tri[t] + nf;
        topo_max[t] = ml;
        // the topology's nodes grouped by level, deepest first (stable in node id)
        std::vector<int> order(nn);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return Lv[a] > Lv[b]; });
        level_node.insert(level_node.end(), order.begin(), order.end());
        std::vector<int> cnt(ml + 1, 0);
        for (int n = 0; n < nn; ++n) cnt[ml - Lv[n]]++;
        int acc = topo_node[t];
        level_start.push_back(acc);
        for (int g = 0; g <= ml; ++g) { acc += cnt[g]; level_start.push_back(acc); }
        topo_level[t + 1] = topo_level[t] + ml + 2;
    }
    std::vector<int> env_node(N), env_face(N);
    int64_t total = 0;
    std::vector<float> amin, amax;
    for (int e = 0; e < N; ++e) {
        env_node[e] = (int)total;
        env_face[e] = c->env_face_start[e];
        const int t = env_topo[e];
        total += topo_node[t + 1] - topo_node[t];
        amin.insert(amin.end(), tmin[t].begin(), tmin[t].end());
        amax.insert(amax.end(), tmax[t].begin(), tmax[t].end());
    }
    if (total >= (1ll << 31)) return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_attach_render: more than 2^31 BVH nodes");
    // point -> incident faces in ascending face id, for the deterministic normal gather
    std::vector<int> pstart(P + 1, 0), pface(3 * (size_t)Fv);
    for (int64_t k = 0; k < 3 * Fv; ++k) pstart[c->faces[k] + 1]++;
    for (int64_t p = 0; p < P; ++p) pstart[p + 1] += pstart[p];
    {
        std::vector<int> fill(pstart.begin(), pstart.end() - 1);
        for (int64_t f = 0; f < Fv; ++f)
            for (int k = 0; k < 3; ++k) pface[fill[c->faces[3 * f + k]]++] = (int)f;
    }
    int32_t st = FFSRL_OK;
    auto chk = [&](int32_t r) { if (r && !st) st = r; };
    ffsrl_bvh& b = h->bvh;
    b.num_envs = N;
    b.num_topologies = M;
    chk(upload_c(h, &b.env_topology, env_topo.data(), N, true));
    chk(upload_c(h, &b.env_node_offset, env_node.data(), N, true));
    chk(upload_c(h, &b.env_face_offset, env_face.data(), N, true));
    chk(upload_c(h, &b.topo_node_offset, topo_node.data(), M + 1, true));
    chk(upload_c(h, &b.topo_tri_offset, topo_tri.data(), M + 1, true));
    chk(upload_c(h, &b.topo_max_level, topo_max.data(), M, true));
    chk(upload_c(h, &b.left_node, left.data(), (int64_t)left.size(), true));
    chk(upload_c(h, &b.first_tri_id, first.data(), (int64_t)first.size(), true));
    chk(upload_c(h, &b.tri_count, count.data(), (int64_t)count.size(), true));
    chk(upload_c(h, &b.level, level.data(), (int64_t)level.size(), true));
    chk(upload_c(h, &b.tri_id, tri.data(), (int64_t)tri.size(), true));
    chk(upload(h, &b.aabb_min, amin.data(), (int64_t)amin.size(), true));
    chk(upload(h, &b.aabb_max, amax.data(), (int64_t)amax.size(), true));
    chk(upload_c(h, &b.level_node, level_node.data(), (int64_t)level_node.size(), true));
    chk(upload_c(h, &b.level_start, level_start.data(), (int64_t)level_start.size(), true));
    chk(upload_c(h, &b.topo_level_offset, topo_level.data(), M + 1, true));
    float* node_box = nullptr;
    float* tri_pos = nullptr;
    chk(upload(h, &node_box, (const float*)nullptr, 8 * total, true));
    chk(upload(h, &tri_pos, (const float*)nullptr, 12 * Fv, true));
    b.node_box = node_box;
    b.tri_pos = tri_pos;
    b.total_env_nodes = (int32_t)total;
    b.total_topology_nodes = topo_node[M];
    b.max_level = *std::max_element(topo_max.begin(), topo_max.end());
    ffsrl_render& r = h->render;
    r.num_envs = N;
    r.resolution = c->resolution;
    r.num_vis_points = (int32_t)P;
    r.num_vis_faces = (int32_t)Fv;
    chk(upload(h, &h->vis_point, c->points, 3 * P, true));
    r.vis_point = h->vis_point;
    chk(upload_c(h, &r.vis_face, c->faces, 3 * Fv, true));
    chk(upload_c(h, &r.vis_point_color, c->colors, 3 * P, true));
    chk(upload(h, &r.normal_sum, (const float*)nullptr, 3 * P, true));
    chk(upload(h, &r.vertex_normal, (const float*)nullptr, 3 * P, true));
    chk(upload_c(h, &r.point_face_start, pstart.data(), P + 1, true));
    chk(upload_c(h, &r.point_face, pface.data(), 3 * Fv, true));
    r.camera_tan = c->camera_tan;
    r.camera_aspect = c->camera_aspect;
    r.num_lights = c->num_lights;
    chk(upload_c(h, &r.light_dir, c->light_dir, 3ll * c->num_lights, false));
    chk(upload_c(h, &r.light_intensity, c->light_intensity, c->num_lights, false));
    chk(upload(h, &r.error_flag, (const int32_t*)nullptr, 1, true));
    chk(upload_c(h, &r.env_point_start, c->env_point_start, N + 1, true));
    r.render_mode = c->render_mode;
    h->num_map = c->num_map;
    chk(upload_c(h, &h->point_to_vertex, c->point_to_vertex, 2ll * c->num_map, false));
    if (st) {
        // give back what this call allocated, so a retried attach does not accumulate them
        for (size_t k = owned0; k < h->owned.size(); ++k) cudaFree(h->owned[k]);
        h->owned.resize(owned0);
        h->bvh = ffsrl_bvh{};
        h->render = ffsrl_render{};
        h->vis_point = nullptr;
        h->point_to_vertex = nullptr;
        return fail(st, std::string("ffsrl_attach_render: upload: ") + ffsrl_last_error());
    }
    h->has_render = true;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_render_handle(ffsrl_handle* h, const float* camera_pos, const float* camera_rot,
                                       int32_t num_cameras, float* color, float* depth, void* stream) {
    if (!h || !h->has_render || !camera_pos || !camera_rot || (num_cameras != 1 && num_cameras != h->dev.num_envs))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render_handle: no render attached, or bad cameras");
    int32_t e;
    if (h->num_map > 0 &&
        (e = ffsrl_remap(h->vis_point, h->dev.vertex, h->point_to_vertex, h->num_map, stream)))
        return e;
    if ((e = ffsrl_bvh_refit_fused(&h->bvh, h->vis_point, h->render.vis_face, stream))) return e;
    ffsrl_render r = h->render;
    r.num_cameras = num_cameras;
    r.camera_pos = camera_pos;
    r.camera_rot = camera_rot;
    r.color = color;
    r.depth = depth;
    return ffsrl_render_fused(&r, &h->bvh, stream);
}

extern "C" int32_t ffsrl_render_handle_check(ffsrl_handle* h, void* stream) {
    if (!h || !h->has_render) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_render_handle_check: no render attached");
    cudaStream_t s = (cudaStream_t)stream;
    int32_t flag = 0;
    FFSRL_CUDA_TRY(cudaMemcpyAsync(&flag, h->render.error_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FFSRL_CUDA_TRY(cudaStreamSynchronize(s));
    if (flag == 0) return FFSRL_OK;
    FFSRL_CUDA_TRY(cudaMemsetAsync(h->render.error_flag, 0, sizeof(int32_t), s));
    FFSRL_CUDA_TRY(cudaStreamSynchronize(s));
    return fail(flag == FFSRL_ERR_STACK_OVERFLOW ? FFSRL_ERR_STACK_OVERFLOW : FFSRL_ERR_CUDA,
                "ffsrl_render_handle: a ray exhausted its BVH traversal stack since the last check");
}
