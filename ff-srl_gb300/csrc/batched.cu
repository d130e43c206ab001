// batched.cu -- the env-resident batched step: plan builder (host) and the fast-form
// instantiations of the kernel (batched_kernel.cuh).  This unit is compiled with
// multiply-add contraction and approximate division; the reference-arithmetic
// instantiations live in batched_ref.cu and the accumulation-study and float64 ones in
// batched_study.cu, which are compiled without contraction and with IEEE division and
// square root.
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
#include "batched_kernel.cuh"

namespace ffsrl {

using namespace bk;

kern_f pick_fast_fixed(int block, int mode, int prefetch, unsigned flags) {
    if (flags == kLiverFlags && mode == 0 && prefetch != 2) {
        if (block == 256) return k_batched<AccFixed, 256, 0, false, kLiverFlags, false>;
        if (block == 512) return k_batched<AccFixed, 512, 0, false, kLiverFlags, false>;
        if (block == 640) return k_batched<AccFixed, 640, 0, false, kLiverFlags, false>;
        if (block == 768) return k_batched<AccFixed, 768, 0, false, kLiverFlags, false>;
        if (block == 1024) return k_batched<AccFixed, 1024, 0, false, kLiverFlags, false>;
    }
    if (flags == kLiverFlags && mode == 0 && prefetch == 2) {
        if (block == 512) return k_batched<AccFixed, 512, 0, true, kLiverFlags, false>;
        if (block == 640) return k_batched<AccFixed, 640, 0, true, kLiverFlags, false>;
        return nullptr;
    }
    if (prefetch == 2) {
        if (mode == 0 && block == 512) return k_batched<AccFixed, 512, 0, true, 0, false>;
        if (mode == 0 && block == 640) return k_batched<AccFixed, 640, 0, true, 0, false>;
        return nullptr;
    }
#define PK(B, M) if (block == B && mode == M) return k_batched<AccFixed, B, M, false, 0, false>;
    PK(128, 0) PK(256, 0) PK(512, 0) PK(640, 0) PK(768, 0) PK(1024, 0)
    PK(256, 1) PK(512, 1) PK(1024, 1)
    PK(256, 2) PK(512, 2)
#undef PK
    return nullptr;
}

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
    float2* d_tet_ed2 = nullptr;  // compact fast-form folded edges
    int compact = 0;              // compact fast-form tet records (48 bytes a tet)
    unsigned* d_edge_idx = nullptr; float2* d_edge_la = nullptr; uint2* d_tri_idx = nullptr;
    int* d_work = nullptr; int* d_counters = nullptr; int* d_status = nullptr;
    unsigned char* d_scratch = nullptr;
    double* d_state64 = nullptr;  // x, v, xp in double for precision 64
    int* d_cnt0 = nullptr;        // static per-vertex contribution counts
    int* d_tet_orig = nullptr;    // record -> model tet id
    int* d_edge_orig = nullptr;   // record -> model edge id
    uint2* d_conn_idx = nullptr; float4* d_conn_bar = nullptr; unsigned char* d_conn_vert = nullptr;
    long long* d_pend = nullptr; int* d_pcnt = nullptr;  // pending connector corrections, kept between steps
    unsigned long long* d_wide = nullptr;  // fixed-point side accumulator [3V], zero between uses
    float4* d_nhd = nullptr;               // reference Neo-Hookean tables: Dm^-1, 3 float4 per tet
    float bound = 1.0f;                    // scaled magnitude one term may take on the 32-bit path
    int arith = FFSRL_ARITH_REFERENCE;     // FFSRL_ARITH_*
    int accum = FFSRL_ACC_FIXED;           // FFSRL_ACC_*
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
    cudaFree(b->d_wide); cudaFree(b->d_nhd); cudaFree(b->d_tet_ed2);
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

// The float32 kernel of a plan's arithmetic and accumulation for a block size, shared-
// memory mode and record prefetch, or null when there is no such instantiation
kern_f kernel_f(const ffsrl_batch* b, int block, int mode, int prefetch) {
    if (b->accum != FFSRL_ACC_FIXED) return prefetch ? nullptr : pick_ref_study(b->accum, block, mode);
    if (b->arith == FFSRL_ARITH_FAST) return pick_fast_fixed(block, mode, prefetch, b->params.flags);
    return pick_ref_fixed(block, mode, prefetch, b->params.flags);
}
const void* kernel_ptr(const ffsrl_batch* b, int block, int mode, int prefetch) {
    if (b->precision == 64) return prefetch ? nullptr : (const void*)pick_ref_f64(block, mode);
    return (const void*)kernel_f(b, block, mode, prefetch);
}
// Shared memory per block and global scratch per block of the plan's storage policy
size_t plan_smem(const ffsrl_batch* b, int mode, int nv) {
    if (b->precision == 64) return smem_bytes<AccF64>(mode, nv);
    if (b->accum == FFSRL_ACC_KAHAN) return smem_bytes<AccKahan>(mode, nv);
    if (b->accum == FFSRL_ACC_ATOMIC) return smem_bytes<AccAtomic>(mode, nv);
    return smem_bytes<AccFixed>(mode, nv);
}
size_t plan_scratch(const ffsrl_batch* b, int mode, int nv) {
    if (b->precision == 64) return scratch_bytes<AccF64>(mode, nv);
    if (b->accum == FFSRL_ACC_KAHAN) return scratch_bytes<AccKahan>(mode, nv);
    if (b->accum == FFSRL_ACC_ATOMIC) return scratch_bytes<AccAtomic>(mode, nv);
    return scratch_bytes<AccFixed>(mode, nv);
}

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
    D.cnt0 = b->d_cnt0; D.tet_orig = b->d_tet_orig; D.edge_orig = b->d_edge_orig;
    D.nhd = b->d_nhd; D.wide = b->d_wide; D.bound = b->bound;
    D.tet_ed = b->d_tet_ed; D.tet_ed2 = b->d_tet_ed2; D.compact = b->compact;
    D.fold = b->d_tet_ed != nullptr || b->d_tet_ed2 != nullptr;
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
    kern_f k = kernel_f(b, c.block, c.mode, c.prefetch);
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
    kern_d k = pick_ref_f64(c.block, c.mode);
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
    D.cnt0 = F.cnt0; D.tet_orig = F.tet_orig; D.edge_orig = F.edge_orig;
    D.nhd = F.nhd; D.wide = F.wide; D.bound = F.bound; D.pend = nullptr; D.pcnt = nullptr;
    D.conn_idx = nullptr; D.conn_bar = nullptr; D.conn_vert = nullptr;
    D.tet_ed = F.tet_ed; D.tet_ed2 = nullptr; D.compact = 0; D.fold = F.fold;
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
    if (b->precision == 64 || b->accum != FFSRL_ACC_FIXED) {
        // the float64 and accumulation-study builds have fewer block sizes: take the
        // nearest one at or above the request that exists
        if (!kernel_ptr(b, block, c.mode, c.prefetch))
            for (int alt : {256, 512, 1024})
                if (alt >= block && kernel_ptr(b, alt, c.mode, c.prefetch)) { block = alt; break; }
        if (!kernel_ptr(b, block, c.mode, c.prefetch)) block = 256;
    }
    if (c.mode == 1 && block < 256) block = 256;
    if (c.mode == 2 && block > 512) block = 512;
    const void* kfn = kernel_ptr(b, block, c.mode, c.prefetch);
    if (!kfn) return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch: no kernel for block " + std::to_string(block) +
                                                     " in mode " + std::to_string(c.mode));
    {
        // the kernel's static shared memory counts against the default 48 KB too, so a
        // class just under 48 KB of dynamic memory needs the opt-in as well; several
        // classes may share one instantiation: allow the whole budget
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
    int arith = FFSRL_ARITH_REFERENCE, accum = FFSRL_ACC_FIXED;
    if (opts) {
        block_override = opts->block_threads;
        arith = opts->arithmetic;
        accum = opts->accumulation;
        if (opts->precision != 0 && opts->precision != 32 && opts->precision != 64)
            return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: precision must be 32 or 64");
        if (opts->precision == 64) precision = 64;
    }
    if (arith != FFSRL_ARITH_REFERENCE && arith != FFSRL_ARITH_FAST)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: unknown arithmetic");
    if (accum != FFSRL_ACC_FIXED && accum != FFSRL_ACC_KAHAN && accum != FFSRL_ACC_ATOMIC)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: unknown accumulation");
    if (precision == 64 && accum != FFSRL_ACC_FIXED)
        return fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_batch_create: the float64 build sums in double; leave "
                                                "accumulation at its default");
    if (arith == FFSRL_ARITH_FAST && (precision == 64 || accum != FFSRL_ACC_FIXED))
        return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch_create: the fast arithmetic exists for the float32 "
                                           "fixed-point step only");
    const bool conn = (p->flags & FFSRL_CONNECTORS) && hm->num_connectors > 0;
    if (conn && (precision == 64 || accum != FFSRL_ACC_FIXED || !hm->connector_vertex_id ||
                 !hm->connector_triangle_id || !hm->connector_tri_bar || !hm->connector_rest_dist))
        return fail(FFSRL_ERR_UNSUPPORTED, "ffsrl_batch_create: connectors need the float32 fixed-point step and "
                                           "all four connector arrays");
    ffsrl_batch* b = new ffsrl_batch();
    b->num_envs = N;
    b->params = *p;
    b->dm = *dmod;
    b->precision = precision;
    b->arith = precision == 64 ? FFSRL_ARITH_REFERENCE : arith;
    b->accum = accum;
    const bool ex = b->arith == FFSRL_ARITH_REFERENCE;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&b->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (b->sm_count <= 0 || b->max_smem <= 0) { free_batch(b); return fail(FFSRL_ERR_CUDA, "ffsrl_batch_create: no device"); }
    // the kernels' static shared memory (block-wide scalars and the instrument) comes off
    // the per-block opt-in limit; budget dynamic shared memory below that
    size_t static_smem = 0;
    {
        const void* probes[] = {(const void*)pick_fast_fixed(1024, 0, 0, 0), (const void*)pick_fast_fixed(512, 1, 0, 0),
                                (const void*)pick_ref_fixed(1024, 0, 0, 0), (const void*)pick_ref_study(FFSRL_ACC_KAHAN, 256, 0),
                                (const void*)pick_ref_f64(256, 0)};
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
    std::vector<float4> nh0, nh1, nhd;  // fast form: M tables; reference form: Dm^-1 (3 per tet)
    std::vector<float> tet_vs;
    const bool nh = (p->flags & FFSRL_NEOHOOKEAN) != 0;
    const bool xv = (p->flags & FFSRL_VOLUME_XPBD) != 0;
    if (nh && !hm->tetrahedron_dm_inv) { free_batch(b); return fail(FFSRL_ERR_INVALID_ARGUMENT, "Neo-Hookean needs tetrahedron_dm_inv"); }
    if (xv && (!hm->xpbd_rest_volume || !dmod->tetrahedron_lambda)) { free_batch(b); return fail(FFSRL_ERR_INVALID_ARGUMENT, "XPBD volume needs xpbd_rest_volume and lambdas"); }
    if ((p->flags & FFSRL_DISTANCE_XPBD) && !dmod->edge_lambda) { free_batch(b); return fail(FFSRL_ERR_INVALID_ARGUMENT, "XPBD distance needs edge_lambda"); }
    if (nh && !ex) { nh0.resize(T); nh1.resize(T); }
    if (nh && ex) nhd.resize(3 * T);
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
            if (nh && ex) {
                // Dm^-1 as stored (row-major), read by the reference-form kernel as the
                // reference reads it
                const float* f = hm->tetrahedron_dm_inv + 9ll * t;
                nhd[3 * t] = make_float4(f[0], f[1], f[2], f[3]);
                nhd[3 * t + 1] = make_float4(f[4], f[5], f[6], f[7]);
                nhd[3 * t + 2] = make_float4(f[8], 0.0f, 0.0f, 0.0f);
            }
            if (nh && !ex) {
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
                   rng_eq(nhd, 3 * a.t0, 3 * c.t0, 3 * a.nt) &&
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

    // ---- fixed-point scale, per env: one unit ~ a quarter float ulp of the env's largest
    // coordinate, so an env's sums (hence its bits) do not depend on the other envs of the
    // model.  A term on the 32-bit path stays below 2^31 / (terms + 1), so a per-vertex sum
    // cannot leave int32; larger terms take the exact 64-bit side path. ----
    for (int e = 0; e < N; ++e) {
        double mx = 1e-30;
        for (int64_t i = 3ll * env[e].v0; i < 3ll * (env[e].v0 + env[e].nv); ++i)
            mx = std::max(mx, (double)std::fabs(hm->vertex[i]));
        int e2 = 0;
        std::frexp(mx, &e2);  // mx < 2^e2
        const int k = std::max(-100, std::min(100, 26 - e2));
        env[e].sc = std::ldexp(1.0f, k);
        env[e].inv = std::ldexp(1.0f, -k);
    }
    b->bound = std::ldexp(1.0f, 31) / (float)(max_terms + 1);

    // ---- fold distance constraints into tets: each edge is solved by one tet that holds
    // both its vertices, inside that tet's thread, so its correction joins the tet's four
    // accumulator updates.  A tet takes at most two edges; its vertices are reordered by an
    // even permutation (same orientation, Neo-Hookean tables recomputed for the new order)
    // so that the edges sit at A-B, and C-D or A-C.  Edges no tet can take stay in the
    // edge loop.  Not with XPBD distance (per-edge multipliers), so edge records keep their
    // model order otherwise. ----
    std::vector<float4> tet_ed;
    // fold class, fast form: 0 none, 1 A-B, 2 A-B + C-D, 3 A-B + A-C; reference form: a bit
    // set of A-B (1), C-D (2), A-C (4)
    std::vector<unsigned char> tet_cls(T, 0);
    const bool fold = (fl & FFSRL_DISTANCE) && !(fl & FFSRL_DISTANCE_XPBD) &&
                      (fl & (FFSRL_VOLUME | FFSRL_VOLUME_XPBD | FFSRL_NEOHOOKEAN)) && T > 0 && E > 0;
    // fast form with Neo-Hookean and folded edges: 48-byte tet records (see below)
    const bool compact = !ex && nh && fold;
    b->compact = compact ? 1 : 0;
    if (fold) {
        tet_ed.assign(T, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        std::vector<unsigned> n_edge_idx;
        std::vector<float2> n_edge_la;
        std::vector<int> adj_start, adj;
        std::vector<int> owned_n(T, 0), owned(2 * T, -1);
        std::vector<int> ex_slot(2 * T, 0);  // reference form: 1 A-B, 2 C-D, 3 A-C
        for (int e = 0; e < N; ++e) {
            EnvRec& r = env[e];
            if (dup_of[e] >= 0) {
                const EnvRec& src = env[dup_of[e]];
                std::copy(tet_idx.begin() + src.t0, tet_idx.begin() + src.t0 + r.nt, tet_idx.begin() + r.t0);
                std::copy(tet_ed.begin() + src.t0, tet_ed.begin() + src.t0 + r.nt, tet_ed.begin() + r.t0);
                std::copy(tet_cls.begin() + src.t0, tet_cls.begin() + src.t0 + r.nt, tet_cls.begin() + r.t0);
                if (nh && !ex) {
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
                if (compact && la.y != 1.0f) {  // compact records fold fully active edges only
                    n_edge_idx.push_back(edge_idx[k]);
                    n_edge_la.push_back(la);
                    continue;
                }
                int best = -1, best_slot = 0;
                for (int j = adj_start[a]; j < adj_start[a + 1]; ++j) {
                    const int t = adj[j];
                    if (owned_n[t] >= 2) continue;
                    uint2 ix = tet_idx[t];
                    int l[4] = {(int)(ix.x & 0xffff), (int)(ix.x >> 16), (int)(ix.y & 0xffff), (int)(ix.y >> 16)};
                    if (l[0] != c && l[1] != c && l[2] != c && l[3] != c) continue;
                    int slot = 0;
                    if (ex) {
                        // reference form: the tet keeps its vertex order, so the edge must sit at
                        // corners A-B (first slot), or C-D / A-C (second slot), and its slot be free
                        int i = 0, q = 0;
                        while (l[i] != a) ++i;
                        while (l[q] != c) ++q;
                        const int lo = std::min(i, q), hi = std::max(i, q);
                        if (lo == 0 && hi == 1) slot = 1;
                        else if (lo == 2 && hi == 3) slot = 2;
                        else if (lo == 0 && hi == 2) slot = 3;
                        else continue;
                        bool taken = false;
                        for (int m = 0; m < owned_n[t]; ++m) {
                            const int os = ex_slot[2 * t + m];
                            if ((os == 1) == (slot == 1)) taken = true;
                        }
                        if (taken) continue;
                    }
                    if (best < 0 || owned_n[t] < owned_n[best]) { best = t; best_slot = slot; }
                }
                if (best >= 0) {
                    ex_slot[2 * best + owned_n[best]] = best_slot;
                    owned[2 * best + owned_n[best]++] = k;
                } else {
                    n_edge_idx.push_back(edge_idx[k]);
                    n_edge_la.push_back(la);
                }
            }
            // reference form: record each owning tet's edges in place
            if (ex) {
                for (int t = r.t0; t < r.t0 + r.nt; ++t) {
                    float4 ed = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    unsigned char cls = 0;
                    for (int m = 0; m < owned_n[t]; ++m) {
                        const float2 la = edge_la[owned[2 * t + m]];
                        const int slot = ex_slot[2 * t + m];
                        if (slot == 1) { ed.x = la.x; ed.y = la.y; cls |= 1; }
                        else if (slot == 2) { ed.z = la.x; ed.w = la.y; cls |= 2; }
                        else { ed.z = -la.x; ed.w = la.y; cls |= 4; }
                    }
                    tet_ed[t] = ed;
                    tet_cls[t] = cls;
                }
                r.e0 = ne_new0;
                r.ne = (int)n_edge_idx.size() - ne_new0;
                continue;
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
                [&](int t) { return col[t] * 8 + tet_cls[r.t0 + t]; });
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
        if (!nhd.empty()) {
            auto c = nhd;
            for (size_t i = 0; i < tet_orig.size(); ++i)
                for (int k = 0; k < 3; ++k) nhd[3 * i + k] = c[3 * (size_t)tet_orig[i] + k];
        }
        permute(tet_vs, tet_orig); permute(tet_ed, tet_orig); permute(edge_idx, edge_orig); permute(edge_la, edge_orig);
    }

    // ---- compact fast-form records: the rest volume carries the volume constraint's
    // activity in its sign (the constraint runs only for activity 1, and then multiplies by
    // it exactly), so nh1.w holds +-|V0| and the tet needs no (V0, active) pair; 1/|V0| is
    // formed in the kernel.  Folded edges are all fully active, so their slots hold the
    // rest lengths alone, 0 for none. ----
    std::vector<float2> tet_ed2;
    if (compact) {
        tet_ed2.resize(T);
        for (int64_t t = 0; t < T; ++t) {
            const float v0 = std::fabs(tet_va[t].x);
            nh1[t].w = tet_va[t].y == 1.0f ? v0 : -v0;
            const float4 ed = tet_ed[t];
            tet_ed2[t] = make_float2(ed.y != 0.0f ? ed.x : 0.0f, ed.w != 0.0f ? ed.z : 0.0f);
        }
        std::vector<float2>().swap(tet_va);
        std::vector<float4>().swap(tet_ed);
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
                   eq(tet_ed2, a.t0, c.t0, a.nt) &&
                   eq(nhd, 3 * a.t0, 3 * c.t0, 3 * a.nt) &&
                   eq(nh1, a.t0, c.t0, a.nt) && eq(tet_vs, a.t0, c.t0, a.nt) && eq(tet_ed, a.t0, c.t0, a.nt) &&
                   eq(tet_orig, a.t0, c.t0, a.nt) && eq(edge_idx, a.e0, c.e0, a.ne) && eq(edge_la, a.e0, c.e0, a.ne) &&
                   eq(edge_orig, a.e0, c.e0, a.ne) && eq(tri_idx, a.f0, c.f0, a.nf);
        };
        std::vector<uint2> c_tet_idx; std::vector<float2> c_tet_va; std::vector<float4> c_nh0, c_nh1, c_nhd;
        std::vector<float> c_tet_vs; std::vector<float4> c_tet_ed; std::vector<int> c_tet_orig, c_edge_orig;
        std::vector<float2> c_tet_ed2;
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
            app(c_nhd, nhd, 3 * r.t0, 3 * r.nt);
            app(c_tet_ed2, tet_ed2, r.t0, r.nt);
            app(c_nh1, nh1, r.t0, r.nt); app(c_tet_vs, tet_vs, r.t0, r.nt); app(c_tet_ed, tet_ed, r.t0, r.nt);
            app(c_tet_orig, tet_orig, r.t0, r.nt); app(c_edge_idx, edge_idx, r.e0, r.ne);
            app(c_edge_la, edge_la, r.e0, r.ne); app(c_edge_orig, edge_orig, r.e0, r.ne);
            app(c_tri_idx, tri_idx, r.f0, r.nf);
        }
        env = out;
        tet_idx.swap(c_tet_idx); tet_va.swap(c_tet_va); nh0.swap(c_nh0); nh1.swap(c_nh1); nhd.swap(c_nhd);
        tet_ed2.swap(c_tet_ed2);
        tet_vs.swap(c_tet_vs); tet_ed.swap(c_tet_ed); tet_orig.swap(c_tet_orig); edge_idx.swap(c_edge_idx); edge_la.swap(c_edge_la);
        edge_orig.swap(c_edge_orig); tri_idx.swap(c_tri_idx);
    }

    // size classes: mode by fit, then by vertex-count band
    const int bands[] = {192, 384, 768, 1536, 3072, 65536};
    b->env_class.assign(N, -1);
    std::vector<std::vector<int>> members;
    std::vector<int> keys;  // mode*16 + band
    auto mode_for = [&](int nv) {
        if (precision == 64) return plan_smem(b, 0, nv) <= dyn_budget ? 0 : 2;
        if (plan_smem(b, 0, nv) <= dyn_budget) return 0;
        if (plan_smem(b, 1, nv) <= dyn_budget) return 1;
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
        c.smem = plan_smem(b, c.mode, c.max_nv);
        if (p->flags & FFSRL_COLLIDE) {
            // the contact scan reads every surface triangle in every iteration: keep the
            // env's triangles in shared memory when they fit
            int max_nf = 0;
            for (int e : mem) max_nf = std::max(max_nf, env[e].nf);
            const size_t with = ((c.smem + 7) & ~(size_t)7) + 8 * (size_t)max_nf;
            if (max_nf > 0 && with <= dyn_budget) { c.tri_cap = max_nf; c.smem = with; }
        }
        c.scratch_stride = plan_scratch(b, c.mode, c.max_nv);
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
        (st = dalloc(b, &b->d_nhd, nhd.size())) || (st = upload(b->d_nhd, nhd)) ||
        (st = dalloc(b, &b->d_wide, (precision == 32 && accum == FFSRL_ACC_FIXED) ? 3 * (size_t)V : 0)) ||
        (st = dalloc(b, &b->d_tet_vs, tet_vs.size())) || (st = upload(b->d_tet_vs, tet_vs)) ||
        (st = dalloc(b, &b->d_tet_ed, tet_ed.size())) || (st = upload(b->d_tet_ed, tet_ed)) ||
        (st = dalloc(b, &b->d_tet_ed2, tet_ed2.size())) || (st = upload(b->d_tet_ed2, tet_ed2)) ||
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
    if (b->d_wide) FFSRL_CUDA_TRY(cudaMemset(b->d_wide, 0, sizeof(unsigned long long) * 3 * (size_t)V));
    if (conn) {
        FFSRL_CUDA_TRY(cudaMemset(b->d_pend, 0, sizeof(long long) * 3 * (size_t)V));
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
