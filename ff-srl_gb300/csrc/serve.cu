// serve.cu -- continuous-batching server of RL step requests over device-resident envs,
// the C-ABI counterpart of ffsrl.serve.EnvServer.
//
// Each actor owns one environment of a given mesh type; environments live in the slots of
// one batched model, and a slot holds an env of one mesh type.  An actor without a slot is
// admitted into a free slot of its type; if there is none, the least recently used idle
// actor of that type is evicted (its state is copied to host memory and restored when it
// returns).  Requests are served in ticks: a tick takes every ready request and runs, for
// exactly those envs, the reset of those starting a new episode, the tool move (through the
// instrument's kinematic chain when it has one), grasp changes, one batched step, the
// visual-point remap, the instrument's visual points, the BVH refit and the ray-cast; then
// each env's result (drag-point position and contact count) is copied to pinned host
// memory.  Lanes -- each with its own stream, staging and the plan's own work lists -- let
// a tick start while earlier ones are still on the GPU.  Each env's result depends only on
// its own inputs, so it is the same in any mix of envs.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>
#include "ffsrl_internal.h"

namespace ffsrl {
namespace {

// result of env ids[i]: its drag point (tip entry 3) and its contact count
__global__ void k_results(const float* __restrict__ tip, const int* __restrict__ incol, const int* __restrict__ ids,
                          int n, float* __restrict__ res) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    long long e = ids[i];
    long long o = 3 * (4 * e + 3);
    res[4 * i] = tip[o];
    res[4 * i + 1] = tip[o + 1];
    res[4 * i + 2] = tip[o + 2];
    res[4 * i + 3] = (float)incol[e];
}

struct Req {
    int actor;
    float disp[3];
    int clamp, reset;
    int64_t tag;
};

struct Snapshot {
    std::vector<float> vertex, velocity, drag, base, tip, xform;
    int incol = 0;
};

struct ServeLane {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    // pinned staging and device copies: env ids, displacements, resets, grasp changes, results
    int* h_ids = nullptr; float* h_disp = nullptr; int* h_rst = nullptr; int* h_gids = nullptr; int* h_gclamp = nullptr;
    float* h_res = nullptr;
    int* d_ids = nullptr; float* d_disp = nullptr; int* d_rst = nullptr; int* d_gids = nullptr; int* d_gclamp = nullptr;
    float* d_res = nullptr;
    std::vector<Req> batch;
};

}  // namespace
}  // namespace ffsrl

using namespace ffsrl;

struct ffsrl_server {
    ffsrl_server_config cfg{};
    ffsrl_model model{};
    ffsrl_bvh bvh{};
    ffsrl_render render{};
    std::vector<int> slot_mesh, actor_mesh, slot_actor, actor_slot, actor_clamp, vstart;
    std::vector<int64_t> last_used;
    std::vector<char> in_flight;
    std::vector<std::vector<int>> free;  // per mesh type, popped from the back
    std::unordered_map<int, Snapshot> snapshots;
    std::deque<Req> pending;
    std::vector<ServeLane> lanes;
    int64_t clock = 0, admissions = 0, evictions = 0;
};

namespace {

int32_t lane_alloc(ServeLane& L, int n) {
    FFSRL_CUDA_TRY(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    FFSRL_CUDA_TRY(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
    FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_ids, sizeof(int) * n, cudaHostAllocDefault));
    FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_disp, sizeof(float) * 3 * n, cudaHostAllocDefault));
    FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_rst, sizeof(int) * n, cudaHostAllocDefault));
    FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_gids, sizeof(int) * n, cudaHostAllocDefault));
    FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_gclamp, sizeof(int) * n, cudaHostAllocDefault));
    FFSRL_CUDA_TRY(cudaHostAlloc((void**)&L.h_res, sizeof(float) * 4 * n, cudaHostAllocDefault));
    FFSRL_CUDA_TRY(cudaMalloc((void**)&L.d_ids, sizeof(int) * n));
    FFSRL_CUDA_TRY(cudaMalloc((void**)&L.d_disp, sizeof(float) * 3 * n));
    FFSRL_CUDA_TRY(cudaMalloc((void**)&L.d_rst, sizeof(int) * n));
    FFSRL_CUDA_TRY(cudaMalloc((void**)&L.d_gids, sizeof(int) * n));
    FFSRL_CUDA_TRY(cudaMalloc((void**)&L.d_gclamp, sizeof(int) * n));
    FFSRL_CUDA_TRY(cudaMalloc((void**)&L.d_res, sizeof(float) * 4 * n));
    return FFSRL_OK;
}

void lane_free(ServeLane& L) {
    if (L.stream) cudaStreamSynchronize(L.stream);
    cudaFreeHost(L.h_ids); cudaFreeHost(L.h_disp); cudaFreeHost(L.h_rst); cudaFreeHost(L.h_gids);
    cudaFreeHost(L.h_gclamp); cudaFreeHost(L.h_res);
    cudaFree(L.d_ids); cudaFree(L.d_disp); cudaFree(L.d_rst); cudaFree(L.d_gids); cudaFree(L.d_gclamp);
    cudaFree(L.d_res);
    if (L.done) cudaEventDestroy(L.done);
    if (L.stream) cudaStreamDestroy(L.stream);
    L = ServeLane{};
}

// range of slot s's vertices
void vrange(const ffsrl_server* S, int s, long long& v0, long long& nv) {
    v0 = S->vstart[s];
    nv = S->vstart[s + 1] - S->vstart[s];
}

int32_t evict(ffsrl_server* S, int a, cudaStream_t st) {
    const int s = S->actor_slot[a];
    long long v0, nv;
    vrange(S, s, v0, nv);
    Snapshot snap;
    snap.vertex.resize(3 * nv); snap.velocity.resize(3 * nv); snap.drag.resize(nv);
    snap.base.resize(12); snap.tip.resize(12);
    const ffsrl_model& m = S->model;
    FFSRL_CUDA_TRY(cudaMemcpyAsync(snap.vertex.data(), m.vertex + 3 * v0, 12 * nv, cudaMemcpyDeviceToHost, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync(snap.velocity.data(), m.velocity + 3 * v0, 12 * nv, cudaMemcpyDeviceToHost, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync(snap.drag.data(), m.active_drag_constraint + v0, 4 * nv, cudaMemcpyDeviceToHost, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync(snap.base.data(), m.laparoscope_base + 12ll * s, 48, cudaMemcpyDeviceToHost, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync(snap.tip.data(), m.laparoscope_tip + 12ll * s, 48, cudaMemcpyDeviceToHost, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync(&snap.incol, m.laparoscope_in_collision + s, 4, cudaMemcpyDeviceToHost, st));
    if (S->cfg.xform) {
        snap.xform.resize(112);
        FFSRL_CUDA_TRY(cudaMemcpyAsync(snap.xform.data(), S->cfg.xform + 112ll * s, 448, cudaMemcpyDeviceToHost, st));
    }
    FFSRL_CUDA_TRY(cudaStreamSynchronize(st));
    S->snapshots[a] = std::move(snap);
    S->actor_slot[a] = -1;
    S->slot_actor[s] = -1;
    S->free[S->slot_mesh[s]].push_back(s);
    ++S->evictions;
    return FFSRL_OK;
}

// the slot's env at rest, the instrument at its initial pose, no grasp (on stream st)
int32_t rest_state(ffsrl_server* S, int s, cudaStream_t st) {
    long long v0, nv;
    vrange(S, s, v0, nv);
    const ffsrl_model& m = S->model;
    const ffsrl_server_config& c = S->cfg;
    FFSRL_CUDA_TRY(cudaMemcpyAsync(m.vertex + 3 * v0, c.initial_vertex + 3 * v0, 12 * nv, cudaMemcpyDeviceToDevice, st));
    FFSRL_CUDA_TRY(cudaMemsetAsync(m.velocity + 3 * v0, 0, 12 * nv, st));
    FFSRL_CUDA_TRY(cudaMemsetAsync((void*)(m.active_drag_constraint + v0), 0, 4 * nv, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)(m.laparoscope_base + 12ll * s), c.initial_base + 12ll * s, 48,
                                   cudaMemcpyDeviceToDevice, st));
    FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)(m.laparoscope_tip + 12ll * s), c.initial_tip + 12ll * s, 48,
                                   cudaMemcpyDeviceToDevice, st));
    FFSRL_CUDA_TRY(cudaMemsetAsync(m.laparoscope_in_collision + s, 0, 4, st));
    if (c.xform)
        FFSRL_CUDA_TRY(cudaMemcpyAsync(c.xform + 112ll * s, c.initial_xform + 112ll * s, 448, cudaMemcpyDeviceToDevice, st));
    return FFSRL_OK;
}

// gives actor a a slot; `busy` (may be null) flags the actors of the tick being formed,
// which may not be evicted for it
int32_t admit(ffsrl_server* S, int a, cudaStream_t st, const char* busy, bool* ok) {
    *ok = false;
    const int mt = S->actor_mesh[a];
    if (S->free[mt].empty()) {
        int victim = -1;
        for (int s = 0; s < S->cfg.num_slots; ++s) {
            const int x = S->slot_actor[s];
            if (S->slot_mesh[s] != mt || x < 0 || S->in_flight[x] || (busy && busy[x])) continue;
            if (victim < 0 || S->last_used[x] < S->last_used[victim]) victim = x;
        }
        if (victim < 0) return FFSRL_OK;
        if (int32_t r = evict(S, victim, st)) return r;
    }
    const int s = S->free[mt].back();
    S->free[mt].pop_back();
    auto it = S->snapshots.find(a);
    if (it != S->snapshots.end()) {
        long long v0, nv;
        vrange(S, s, v0, nv);
        const Snapshot& p = it->second;
        const ffsrl_model& m = S->model;
        // copies from pageable memory: the host buffers may go once the calls return
        FFSRL_CUDA_TRY(cudaMemcpyAsync(m.vertex + 3 * v0, p.vertex.data(), 12 * nv, cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaMemcpyAsync(m.velocity + 3 * v0, p.velocity.data(), 12 * nv, cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)(m.active_drag_constraint + v0), p.drag.data(), 4 * nv,
                                       cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)(m.laparoscope_base + 12ll * s), p.base.data(), 48, cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaMemcpyAsync((void*)(m.laparoscope_tip + 12ll * s), p.tip.data(), 48, cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaMemcpyAsync(m.laparoscope_in_collision + s, &p.incol, 4, cudaMemcpyHostToDevice, st));
        if (S->cfg.xform && !p.xform.empty())
            FFSRL_CUDA_TRY(cudaMemcpyAsync(S->cfg.xform + 112ll * s, p.xform.data(), 448, cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaStreamSynchronize(st));
        S->snapshots.erase(it);
    } else {
        if (int32_t r = rest_state(S, s, st)) return r;
        S->actor_clamp[a] = 0;
    }
    S->actor_slot[a] = s;
    S->slot_actor[s] = a;
    ++S->admissions;
    *ok = true;
    return FFSRL_OK;
}

}  // namespace

extern "C" int32_t ffsrl_server_create(const ffsrl_server_config* c, ffsrl_server** out) {
    if (!out) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_create: out is NULL");
    *out = nullptr;
    if (!c || c->num_slots <= 0 || c->num_actors <= 0 || !c->slot_mesh || !c->actor_mesh || !c->plan || !c->model ||
        !c->bvh || !c->render || !c->initial_vertex || !c->initial_base || !c->initial_tip || !c->grasp_cand_start ||
        !c->grasp_cand || !c->vis_point || !c->point_to_vertex || !c->env_map_start || !c->vis_face ||
        c->lanes < 1 || c->lanes > 2 || (c->xform && (!c->initial_xform || !c->height)) ||
        (c->inst_num_points > 0 && (!c->xform || !c->inst_local_point || !c->inst_point_slot || !c->env_inst_first_point)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_create: missing or inconsistent configuration");
    const ffsrl_model* m = c->model;
    if (m->num_envs != c->num_slots || !m->vertex || !m->velocity || !m->active_drag_constraint ||
        !m->laparoscope_base || !m->laparoscope_tip || !m->laparoscope_in_collision || !m->env_vertex_start)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_create: the model's env count or arrays do not fit");
    int types = 0;
    for (int s = 0; s < c->num_slots; ++s) {
        if (c->slot_mesh[s] < 0) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_create: negative mesh type");
        types = std::max(types, c->slot_mesh[s] + 1);
    }
    for (int a = 0; a < c->num_actors; ++a)
        if (c->actor_mesh[a] < 0 || c->actor_mesh[a] >= types)
            return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_create: an actor's mesh type has no slot");
    auto* S = new ffsrl_server;
    S->cfg = *c;
    S->model = *c->model;
    S->bvh = *c->bvh;
    S->render = *c->render;
    S->cfg.model = &S->model;
    S->cfg.bvh = &S->bvh;
    S->cfg.render = &S->render;
    S->slot_mesh.assign(c->slot_mesh, c->slot_mesh + c->num_slots);
    S->actor_mesh.assign(c->actor_mesh, c->actor_mesh + c->num_actors);
    S->cfg.slot_mesh = S->slot_mesh.data();
    S->cfg.actor_mesh = S->actor_mesh.data();
    S->vstart.resize(c->num_slots + 1);
    if (cudaMemcpy(S->vstart.data(), m->env_vertex_start, sizeof(int) * (c->num_slots + 1), cudaMemcpyDeviceToHost) !=
        cudaSuccess) {
        delete S;
        return fail(FFSRL_ERR_CUDA, "ffsrl_server_create: reading the env vertex ranges");
    }
    S->slot_actor.assign(c->num_slots, -1);
    S->actor_slot.assign(c->num_actors, -1);
    S->actor_clamp.assign(c->num_actors, 0);
    S->last_used.assign(c->num_actors, 0);
    S->in_flight.assign(c->num_actors, 0);
    S->free.resize(types);
    for (int s = c->num_slots - 1; s >= 0; --s) S->free[S->slot_mesh[s]].push_back(s);  // lowest slot first
    S->lanes.resize(c->lanes);
    for (auto& L : S->lanes)
        if (int32_t r = lane_alloc(L, c->num_slots)) {
            for (auto& K : S->lanes) lane_free(K);
            delete S;
            return r;
        }
    *out = S;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_server_destroy(ffsrl_server* S) {
    if (!S) return FFSRL_OK;
    for (auto& L : S->lanes) lane_free(L);
    delete S;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_server_submit(ffsrl_server* S, int32_t actor, const float* disp, int32_t clamp, int32_t reset,
                                       int64_t tag) {
    if (!S || !disp || actor < 0 || actor >= S->cfg.num_actors)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_submit: bad server, actor or displacement");
    Req r;
    r.actor = actor;
    std::memcpy(r.disp, disp, sizeof(r.disp));
    r.clamp = clamp;
    r.reset = reset;
    r.tag = tag;
    S->pending.push_back(r);
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_server_admit(ffsrl_server* S, int32_t actor, int32_t* slot) {
    if (!S || actor < 0 || actor >= S->cfg.num_actors) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_admit");
    if (S->actor_slot[actor] < 0) {
        bool ok = false;
        if (int32_t r = admit(S, actor, S->lanes[0].stream, nullptr, &ok)) return r;
        if (!ok) return fail(FFSRL_ERR_BUSY, "ffsrl_server_admit: every slot of the actor's mesh type is in flight");
        FFSRL_CUDA_TRY(cudaStreamSynchronize(S->lanes[0].stream));
    }
    if (slot) *slot = S->actor_slot[actor];
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_server_evict(ffsrl_server* S, int32_t actor) {
    if (!S || actor < 0 || actor >= S->cfg.num_actors) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_evict");
    if (S->actor_slot[actor] < 0) return FFSRL_OK;
    if (S->in_flight[actor]) return fail(FFSRL_ERR_BUSY, "ffsrl_server_evict: the actor's tick has not been polled");
    return evict(S, actor, S->lanes[0].stream);
}

extern "C" int32_t ffsrl_server_launch(ffsrl_server* S, int32_t max_batch, int32_t* launched) {
    if (!S) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_launch");
    if (launched) *launched = 0;
    int li = -1;
    for (size_t k = 0; k < S->lanes.size(); ++k)
        if (S->lanes[k].batch.empty()) { li = (int)k; break; }
    if (li < 0 || S->pending.empty()) return FFSRL_OK;  // every lane busy or waiting to be polled
    ServeLane& L = S->lanes[li];
    cudaStream_t st = L.stream;
    std::vector<Req> batch;
    std::deque<Req> rest;
    std::vector<char> seen(S->cfg.num_actors, 0);
    for (const Req& r : S->pending) {
        if (S->in_flight[r.actor] || seen[r.actor] || (max_batch > 0 && (int)batch.size() >= max_batch)) {
            rest.push_back(r);
            continue;
        }
        if (S->actor_slot[r.actor] < 0) {
            bool ok = false;
            if (int32_t e = admit(S, r.actor, st, seen.data(), &ok)) return e;
            if (!ok) { rest.push_back(r); continue; }
        }
        seen[r.actor] = 1;
        batch.push_back(r);
    }
    const int n = (int)batch.size();
    if (!n) {
        S->pending.swap(rest);
        return FFSRL_OK;
    }
    const ffsrl_server_config& c = S->cfg;
    const ffsrl_model& m = S->model;
    const int N = c.num_slots;
    int nr = 0, ng = 0;
    for (int i = 0; i < n; ++i) {
        const Req& r = batch[i];
        const int s = S->actor_slot[r.actor];
        L.h_ids[i] = s;
        for (int k = 0; k < 3; ++k) L.h_disp[3 * i + k] = r.disp[k];
        if (r.reset) L.h_rst[nr++] = s;
    }
    for (int i = 0; i < n; ++i) {
        const Req& r = batch[i];
        // a reset opens the grasp; the clamp then closes again below if the request asks
        const int cur = r.reset ? 0 : S->actor_clamp[r.actor];
        if (r.clamp != cur) {
            L.h_gids[ng] = L.h_ids[i];
            L.h_gclamp[ng++] = r.clamp;
        }
    }
    // The queue and the clamp states change only once every launch of the tick has been
    // issued: if one fails, the batch's requests stay queued in their order and the clamp
    // states keep describing the device (launches already issued are not undone).
    auto issue = [&]() -> int32_t {
        FFSRL_CUDA_TRY(cudaMemcpyAsync(L.d_ids, L.h_ids, sizeof(int) * n, cudaMemcpyHostToDevice, st));
        FFSRL_CUDA_TRY(cudaMemcpyAsync(L.d_disp, L.h_disp, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
        int32_t e = FFSRL_OK;
        if (nr) {
            FFSRL_CUDA_TRY(cudaMemcpyAsync(L.d_rst, L.h_rst, sizeof(int) * nr, cudaMemcpyHostToDevice, st));
            e = ffsrl_reset_envs(m.vertex, m.velocity, (float*)m.active_drag_constraint, c.initial_vertex,
                                 (float*)m.laparoscope_base, (float*)m.laparoscope_tip, c.initial_base, c.initial_tip,
                                 m.laparoscope_in_collision, c.xform, c.initial_xform, m.env_vertex_start, L.d_rst, nr,
                                 N, st);
            if (e) return e;
        }
        if (c.xform)  // the effector moves through the instrument's kinematic chain
            e = ffsrl_instrument_cartesian_envs(c.xform, L.d_disp, nullptr, nullptr, (float*)m.laparoscope_base,
                                                (float*)m.laparoscope_tip, c.height, L.d_ids, n, N, st);
        else
            e = ffsrl_move_tool_envs((float*)m.laparoscope_base, (float*)m.laparoscope_tip, L.d_disp, L.d_ids, n, N,
                                     st);
        if (e) return e;
        if (ng) {
            FFSRL_CUDA_TRY(cudaMemcpyAsync(L.d_gids, L.h_gids, sizeof(int) * ng, cudaMemcpyHostToDevice, st));
            FFSRL_CUDA_TRY(cudaMemcpyAsync(L.d_gclamp, L.h_gclamp, sizeof(int) * ng, cudaMemcpyHostToDevice, st));
            if ((e = ffsrl_grasp_nearest_envs(m.vertex, c.grasp_cand_start, c.grasp_cand, m.laparoscope_tip,
                                              L.d_gclamp, c.grasp_radius, (float*)m.active_drag_constraint, L.d_gids,
                                              ng, N, st)))
                return e;
        }
        if ((e = ffsrl_batch_step_envs_lane(c.plan, li, L.h_ids, n, 1, st))) return e;
        if ((e = ffsrl_remap_envs(c.vis_point, m.vertex, c.point_to_vertex, c.env_map_start, L.d_ids, n, N, st)))
            return e;
        if (c.inst_num_points > 0 &&
            (e = ffsrl_instrument_visual_update(c.xform, c.inst_local_point, c.inst_point_slot, c.inst_num_points,
                                                c.vis_point, c.env_inst_first_point, L.d_ids, n, N, st)))
            return e;
        if ((e = ffsrl_bvh_refit_fused_envs(&S->bvh, c.vis_point, c.vis_face, L.d_ids, n, st))) return e;
        if ((e = ffsrl_render_fused_envs(&S->render, &S->bvh, L.d_ids, n, st))) return e;
        k_results<<<grid_for(n, 128), 128, 0, st>>>(m.laparoscope_tip, m.laparoscope_in_collision, L.d_ids, n,
                                                    L.d_res);
        FFSRL_LAUNCH_CHECK("ffsrl_server_launch: results");
        FFSRL_CUDA_TRY(cudaMemcpyAsync(L.h_res, L.d_res, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, st));
        FFSRL_CUDA_TRY(cudaEventRecord(L.done, st));
        return FFSRL_OK;
    };
    if (int32_t e = issue()) return e;
    S->pending.swap(rest);
    for (const Req& r : batch) S->actor_clamp[r.actor] = r.clamp;
    ++S->clock;
    for (const Req& r : batch) {
        S->in_flight[r.actor] = 1;
        S->last_used[r.actor] = S->clock;
    }
    L.batch.swap(batch);
    if (launched) *launched = n;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_server_poll(ffsrl_server* S, int32_t capacity, int64_t* tags, int32_t* actors,
                                     float* results, int32_t* count) {
    if (!S || !count || capacity < 0 || (capacity > 0 && (!tags || !actors || !results)))
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_poll");
    *count = 0;
    for (auto& L : S->lanes) {
        const int n = (int)L.batch.size();
        if (!n || *count + n > capacity) continue;
        cudaError_t q = cudaEventQuery(L.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return cuda_fail(q, "ffsrl_server_poll");
        for (int i = 0; i < n; ++i) {
            const int o = *count + i;
            tags[o] = L.batch[i].tag;
            actors[o] = L.batch[i].actor;
            std::memcpy(results + 4ll * o, L.h_res + 4ll * i, 4 * sizeof(float));
            S->in_flight[L.batch[i].actor] = 0;
        }
        *count += n;
        L.batch.clear();
    }
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_server_stats(const ffsrl_server* S, int64_t* admissions, int64_t* evictions, int32_t* pending,
                                      int32_t* in_flight) {
    if (!S) return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_server_stats");
    if (admissions) *admissions = S->admissions;
    if (evictions) *evictions = S->evictions;
    if (pending) *pending = (int32_t)S->pending.size();
    if (in_flight) {
        int k = 0;
        for (auto& L : S->lanes) k += (int)L.batch.size();
        *in_flight = k;
    }
    return FFSRL_OK;
}
