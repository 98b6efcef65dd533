// uneven.cu -- batches of complex transforms of uneven lengths in one launch.
//
// The reference has no batch API (callers loop over kfft_eval_cpx on the host,
// ext/2d/kfft_cpx2.c:100-104).  Here a batch of `count` sequences packed back
// to back is planned once: one device plan per distinct length (radices up to
// 16, so primes p whose p-1 is 13-smooth use Rader and the rest Bluestein),
// one chain of pass descriptors per sequence with its own workspace slice,
// and a device work queue of (pass, tile) items ordered by dependency level.
// One persistent kernel drains the queue; a tile whose pass depends on an
// earlier pass of the same sequence waits (bounded) for that pass's tile
// counter.  The counter reset and the kernel are recorded in a CUDA graph that
// every call replays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "engine.cuh"
#include "kfft.h"

using namespace kfft;

namespace {
constexpr uint32_t kUnevenMaxPrime = 13;

struct Item {
    uint32_t desc;
    uint32_t tile;
};
}  // namespace

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
    // queue recorded for (in, out)
    const void* g_in = nullptr;
    void* g_out = nullptr;
    void* qmem = nullptr;  // descs | extras | deps | items | counters
    size_t qbytes = 0;
    uint32_t* counters = nullptr;  // head, error, done[ndesc]
    size_t counter_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    uint32_t ndesc = 0, nitems = 0;
    std::mutex mu;
    void drop_queue() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (qmem) {
            cudaFree(qmem);
            account_device_bytes(-int64_t(qbytes));
        }
        qmem = nullptr;
        qbytes = 0;
    }
    ~kfft_plan_uneven() {
        drop_queue();
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

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

// Builds every sequence's pass chain, the dependency table and the level-ordered
// queue, uploads them and records the graph.
bool record(kfft_plan_uneven* P, const vec2_t* in, vec2_t* out) {
    std::vector<PassDesc> all;
    std::vector<int32_t> deps;
    std::vector<uint32_t> level;
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
        used += a256(wb);
        Layout l;
        l.batch = 1;
        l.bs = n;
        const size_t first = all.size();
        if (!build_passes(fp, in + P->offsets[i], l, out + P->offsets[i], l,
                          scale_for(P->flags, n), ws, all))
            return false;
        for (size_t k = first; k < all.size(); ++k) {
            deps.push_back(k == first ? -1 : int32_t(k - 1));
            level.push_back(uint32_t(k - first));
        }
    }
    const uint32_t nd = uint32_t(all.size());
    for (const PassDesc& d : all)
        if (!d.regmode) return false;  // the queue kernel runs register-resident tiles only
    std::vector<Item> items;
    uint32_t smem = 0;
    for (uint32_t d = 0; d < nd; ++d) {
        smem = std::max(smem, all[d].smem_bytes);
        for (uint32_t t = 0; t < all[d].tiles; ++t) items.push_back({d, t});
    }
    // level order (dependencies first), larger tiles first within a level
    std::stable_sort(items.begin(), items.end(), [&](const Item& a, const Item& b) {
        if (level[a.desc] != level[b.desc]) return level[a.desc] < level[b.desc];
        const uint64_t wa = uint64_t(all[a.desc].R) * all[a.desc].C;
        const uint64_t wb = uint64_t(all[b.desc].R) * all[b.desc].C;
        return wa > wb;
    });
    const size_t b_desc = a256(sizeof(PassDesc) * nd);
    const size_t b_extra = a256(pass_extra_bytes() * nd);
    const size_t b_dep = a256(sizeof(int32_t) * nd);
    const size_t b_item = a256(sizeof(Item) * items.size());
    const size_t b_cnt = a256(sizeof(uint32_t) * (nd + 2));
    P->drop_queue();
    P->qbytes = b_desc + b_extra + b_dep + b_item + b_cnt;
    if (cudaMalloc(&P->qmem, P->qbytes) != cudaSuccess) {
        cudaGetLastError();
        P->qmem = nullptr;
        return false;
    }
    account_device_bytes(int64_t(P->qbytes));
    char* q = static_cast<char*>(P->qmem);
    PassDesc* d_desc = reinterpret_cast<PassDesc*>(q);
    void* d_extra = q + b_desc;
    int32_t* d_dep = reinterpret_cast<int32_t*>(q + b_desc + b_extra);
    Item* d_item = reinterpret_cast<Item*>(q + b_desc + b_extra + b_dep);
    P->counters = reinterpret_cast<uint32_t*>(q + b_desc + b_extra + b_dep + b_item);
    P->counter_bytes = sizeof(uint32_t) * (nd + 2);
    std::vector<char> extras(pass_extra_bytes() * nd);
    fill_extras(all.data(), extras.data(), nd);
    cudaStream_t st = cudaStreamPerThread;
    cudaMemcpyAsync(d_desc, all.data(), sizeof(PassDesc) * nd, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_extra, extras.data(), extras.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_dep, deps.data(), sizeof(int32_t) * nd, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_item, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return false;
    P->ndesc = nd;
    P->nitems = uint32_t(items.size());

    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(P->counters, 0, P->counter_bytes, cap);
        launch_persistent(d_desc, d_extra, d_dep, d_item, P->nitems, P->counters,
                          P->counters + 2, P->counters + 1, smem, cap);
        e = cudaStreamEndCapture(cap, &graph);
    }
    count_launch(-1);  // counted on every replay instead
    if (e == cudaSuccess) e = cudaGraphInstantiate(&P->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        P->exec = nullptr;
        return false;
    }
    P->g_in = in;
    P->g_out = out;
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
        if (!record(P, in, out)) return KFFT_RET_BUFFER_FAIL;
    }
    cudaError_t e = cudaGraphLaunch(P->exec, st);
    count_graph_launch();
    count_launch(1);
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
            FftPlan* fp = make_plan(n, sign, P->arena, st, kUnevenMaxPrime);
            if (!fp) return NULL;
            P->plans[n].reset(fp);
        }
        ws += a256(workspace_bytes(*P->plans[n], 1));
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
    if (take_pending_error()) return NULL;
    return P.release();
}

KFFT_API uint64_t kfft_uneven_total(const kfft_plan_uneven* plan) { return plan ? plan->total : 0; }

KFFT_API kfft_return_t kfft_eval_cpx_uneven_async(kfft_plan_uneven* plan, const kfft_cpx* fin,
                                                  kfft_cpx* fout, void* stream) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    std::lock_guard<std::mutex> lk(plan->mu);
    cudaSetDevice(current_device());
    kfft_return_t r = launch(plan, reinterpret_cast<const vec2_t*>(fin),
                             reinterpret_cast<vec2_t*>(fout), static_cast<cudaStream_t>(stream));
    if (take_pending_error()) return KFFT_RET_BUFFER_FAIL;
    return r;
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
    uint32_t err = 0;
    cudaMemcpyAsync(&err, plan->counters + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) note_cuda_error(e);
    if (take_pending_error() || err) return KFFT_RET_BUFFER_FAIL;
    return KFFT_RET_SUCCESS;
}

KFFT_API void kfft_release_uneven(kfft_plan_uneven* plan) { delete plan; }

}  // extern "C"
