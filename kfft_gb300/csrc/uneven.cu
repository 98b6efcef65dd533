// uneven.cu -- batches of complex transforms of uneven lengths.
//
// The reference has no batch API (callers loop over kfft_eval_cpx on the host,
// ext/2d/kfft_cpx2.c:100-104).  Here a batch of `count` sequences packed back
// to back is planned once: one device plan per distinct length, one chain of
// pass descriptors per sequence, each chain with its own slice of workspace.
// Execution is recorded once into a CUDA graph and replayed per call.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "engine.cuh"
#include "kfft.h"

using namespace kfft;

struct kfft_plan_uneven {
    uint32_t flags = 0;
    std::vector<uint32_t> lengths;
    std::vector<uint64_t> offsets;
    uint64_t total = 0;
    DeviceArena arena;
    std::map<uint32_t, std::unique_ptr<FftPlan>> plans;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    void* stage = nullptr;  // host staging: in and out, total points each
    // graph recorded for (in, out)
    const void* g_in = nullptr;
    void* g_out = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t nodes = 0;
    std::mutex mu;
    ~kfft_plan_uneven() {
        if (exec) cudaGraphExecDestroy(exec);
        if (ws) {
            cudaFree(ws);
            account_device_bytes(-int64_t(ws_bytes));
        }
        if (stage) {
            cudaFree(stage);
            account_device_bytes(-int64_t(2 * total * sizeof(vec2_t)));
        }
    }
};

namespace {
real_t scale_for(uint32_t flags, uint32_t n) {
    if (!(flags & KFFT_FLAG_INVERSE) || (flags & KFFT_FLAG_DISABLE_NORM)) return real_t(1);
    return real_t(1.0 / double(n));
}

bool record(kfft_plan_uneven* P, const vec2_t* in, vec2_t* out, cudaStream_t st,
            std::vector<PassDesc>& all) {
    char* base = static_cast<char*>(P->ws);
    size_t used = 0;
    for (size_t i = 0; i < P->lengths.size(); ++i) {
        const uint32_t n = P->lengths[i];
        if (n == 0) continue;
        const FftPlan& fp = *P->plans[n];
        size_t wb = workspace_bytes(fp, 1);
        Workspace ws;
        ws.base = base + used;
        ws.size = wb;
        used += (wb + 255) & ~size_t(255);
        Layout l;
        l.batch = 1;
        l.bs = n;
        if (!build_passes(fp, in + P->offsets[i], l, out + P->offsets[i], l,
                          scale_for(P->flags, n), ws, all))
            return false;
    }
    (void)st;
    return true;
}

bool is_dev(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

kfft_return_t launch(kfft_plan_uneven* P, const vec2_t* in, vec2_t* out, cudaStream_t st) {
    if (!P->exec || P->g_in != in || P->g_out != out) {
        if (P->exec) {
            cudaGraphExecDestroy(P->exec);
            P->exec = nullptr;
        }
        std::vector<PassDesc> all;
        if (!record(P, in, out, st, all)) return KFFT_RET_BUFFER_FAIL;
        cudaStream_t cap;
        if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
            return KFFT_RET_BUFFER_FAIL;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            run_passes(all, cap);
            e = cudaStreamEndCapture(cap, &graph);
        }
        // recording counted the kernels once; they run on every replay instead
        count_launch(-int64_t(all.size()));
        P->nodes = int64_t(all.size());
        if (e == cudaSuccess) e = cudaGraphInstantiate(&P->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) {
            note_cuda_error(e);
            P->exec = nullptr;
            return KFFT_RET_BUFFER_FAIL;
        }
        P->g_in = in;
        P->g_out = out;
    }
    cudaError_t e = cudaGraphLaunch(P->exec, st);
    count_graph_launch();
    count_launch(P->nodes);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        return KFFT_RET_BUFFER_FAIL;
    }
    return KFFT_RET_SUCCESS;
}
}  // namespace

extern "C" {

KFFT_API kfft_plan_uneven* kfft_config_cpx_uneven(uint32_t count, const uint32_t* lengths,
                                                  uint32_t flags) {
    if (!lengths && count) return NULL;
    if (!ensure_device()) return NULL;
    std::unique_ptr<kfft_plan_uneven> P(new kfft_plan_uneven());
    P->flags = flags;
    P->lengths.assign(lengths, lengths + count);
    P->offsets.resize(count);
    const int sign = (flags & KFFT_FLAG_INVERSE) ? +1 : -1;
    cudaStream_t st = cudaStreamPerThread;
    size_t ws = 0;
    for (uint32_t i = 0; i < count; ++i) {
        P->offsets[i] = P->total;
        P->total += lengths[i];
        const uint32_t n = lengths[i];
        if (n == 0) continue;
        if (!P->plans.count(n)) {
            FftPlan* fp = make_plan(n, sign, P->arena, st);
            if (!fp) return NULL;
            P->plans[n].reset(fp);
        }
        ws += (workspace_bytes(*P->plans[n], 1) + 255) & ~size_t(255);
    }
    if (ws) {
        if (cudaMalloc(&P->ws, ws) != cudaSuccess) {
            cudaGetLastError();
            return NULL;
        }
        P->ws_bytes = ws;
        account_device_bytes(int64_t(ws));
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return NULL;
    return P.release();
}

KFFT_API uint64_t kfft_uneven_total(const kfft_plan_uneven* plan) { return plan ? plan->total : 0; }

KFFT_API kfft_return_t kfft_eval_cpx_uneven_async(kfft_plan_uneven* plan, const kfft_cpx* fin,
                                                  kfft_cpx* fout, void* stream) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    std::lock_guard<std::mutex> lk(plan->mu);
    cudaSetDevice(current_device());
    return launch(plan, reinterpret_cast<const vec2_t*>(fin), reinterpret_cast<vec2_t*>(fout),
                  static_cast<cudaStream_t>(stream));
}

KFFT_API kfft_return_t kfft_eval_cpx_uneven(kfft_plan_uneven* plan, const kfft_cpx* fin,
                                            kfft_cpx* fout) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    std::lock_guard<std::mutex> lk(plan->mu);
    cudaSetDevice(current_device());
    cudaStream_t st = cudaStreamPerThread;
    const size_t bytes = sizeof(vec2_t) * plan->total;
    const bool hin = !is_dev(fin), hout = !is_dev(fout);
    const vec2_t* din = reinterpret_cast<const vec2_t*>(fin);
    vec2_t* dout = reinterpret_cast<vec2_t*>(fout);
    if ((hin || hout) && !plan->stage) {
        if (cudaMalloc(&plan->stage, 2 * bytes) != cudaSuccess) {
            cudaGetLastError();
            return KFFT_RET_BUFFER_FAIL;
        }
        account_device_bytes(int64_t(2 * bytes));
    }
    vec2_t* s_in = static_cast<vec2_t*>(plan->stage);
    vec2_t* s_out = s_in ? s_in + plan->total : nullptr;
    if (hin) {
        cudaMemcpyAsync(s_in, fin, bytes, cudaMemcpyHostToDevice, st);
        din = s_in;
    }
    if (hout) dout = s_out;
    kfft_return_t r = launch(plan, din, dout, st);
    if (r != KFFT_RET_SUCCESS) return r;
    if (hout) cudaMemcpyAsync(fout, dout, bytes, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        return KFFT_RET_BUFFER_FAIL;
    }
    return KFFT_RET_SUCCESS;
}

KFFT_API void kfft_release_uneven(kfft_plan_uneven* plan) { delete plan; }

}  // extern "C"
