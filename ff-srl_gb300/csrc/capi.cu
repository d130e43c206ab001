// capi.cu -- library-wide entry points: ABI version, per-thread last error, device info.
#include <cuda_runtime.h>
#include <string>
#include "ffsrl_internal.h"

namespace ffsrl {
namespace {
thread_local std::string g_last_error;
}
int32_t fail(int32_t code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
void clear_error() { g_last_error.clear(); }
}  // namespace ffsrl

extern "C" int32_t ffsrl_abi_version(void) { return FFSRL_ABI_VERSION; }

extern "C" const char* ffsrl_last_error(void) { return ffsrl::g_last_error.c_str(); }

extern "C" int32_t ffsrl_device_info(int32_t* sm_count, int32_t* max_smem_per_block, int32_t* cc_major,
                                     int32_t* cc_minor) {
    int dev = 0, n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        if (sm_count) *sm_count = 0;
        if (max_smem_per_block) *max_smem_per_block = 0;
        if (cc_major) *cc_major = 0;
        if (cc_minor) *cc_minor = 0;
        return ffsrl::fail(FFSRL_ERR_CUDA, "ffsrl_device_info: no CUDA device");
    }
    cudaGetDevice(&dev);
    int v = 0;
    if (sm_count) { cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev); *sm_count = v; }
    if (max_smem_per_block) { cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev); *max_smem_per_block = v; }
    if (cc_major) { cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, dev); *cc_major = v; }
    if (cc_minor) { cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, dev); *cc_minor = v; }
    return FFSRL_OK;
}

// ---- CUDA graphs of library calls (the reference's wp.capture_begin / capture_end /
// capture_launch, bvh.py:442-451, render.py:1108-1112) ----
struct ffsrl_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" int32_t ffsrl_graph_begin(void* stream) {
    if (!stream) return ffsrl::fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_graph_begin: the legacy default stream cannot be captured");
    FFSRL_CUDA_TRY(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_graph_end(void* stream, ffsrl_graph** out) {
    if (!stream || !out) return ffsrl::fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_graph_end");
    *out = nullptr;
    cudaGraph_t g = nullptr;
    FFSRL_CUDA_TRY(cudaStreamEndCapture((cudaStream_t)stream, &g));
    cudaGraphExec_t e = nullptr;
    cudaError_t st = cudaGraphInstantiate(&e, g, 0);
    if (st != cudaSuccess) {
        cudaGraphDestroy(g);
        return ffsrl::cuda_fail(st, "ffsrl_graph_end: instantiate");
    }
    ffsrl_graph* h = new ffsrl_graph;
    h->graph = g;
    h->exec = e;
    *out = h;
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_graph_launch(const ffsrl_graph* g, void* stream) {
    if (!g || !g->exec) return ffsrl::fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_graph_launch");
    FFSRL_CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    return FFSRL_OK;
}

extern "C" int32_t ffsrl_graph_destroy(ffsrl_graph* g) {
    if (!g) return FFSRL_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return FFSRL_OK;
}
