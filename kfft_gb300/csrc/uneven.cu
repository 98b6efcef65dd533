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

// Register tiles of the queue kernel: most points per tile and longest pass
// (build-time knobs; the queue kernel's resident CTAs per SM are
// KFFT_QUEUE_MINBLOCKS).  Tiles of at most 2048 points and passes of at most
// 512, measured on the uneven batch of 3968 sequences: FP32 at four CTAs per
// SM 9.38 ms against 9.96 ms for 4096 / 1024 at three (4096 / 512 at four:
// 10.37 ms; 2048 / 512 at three: 11.48 ms; 1024 / 256 at four: 14.89 ms);
// FP64 at three CTAs per SM 84.1 ms against 100.1 ms for 4096 / 1024 at two
// (2048 / 512 at two: 87.7 ms).
#ifndef KFFT_QUEUE_TILE
#define KFFT_QUEUE_TILE 2048
#endif
#ifndef KFFT_QUEUE_RMAX
#define KFFT_QUEUE_RMAX 512
#endif

namespace {
constexpr uint32_t kUnevenMaxPrime = 13;

// the queue kernel's item record: tile `tile` of pass `desc`, runnable once
// done[dep] reaches `need` (dep < 0: no dependency)
struct Item {
    uint32_t desc;
    uint32_t tile;
    int32_t dep;
    uint32_t need;
};
static_assert(sizeof(Item) == 16, "one 16-byte record per item");
}  // namespace

// One recorded work queue over a range of sequences: descriptors, items and
// counters in device memory, and the graph (counter reset + persistent
// kernel) that replays it for one (in, out) pair.
struct UnevenQueue {
    size_t s0 = 0, s1 = 0;  // sequences [s0, s1)
    uint64_t p0 = 0, p1 = 0;  // their points [p0, p1)
    const void* g_in = nullptr;
    void* g_out = nullptr;
    void* qmem = nullptr;  // descs | extras | items | counters
    size_t qbytes = 0;
    uint32_t* counters = nullptr;  // head, error, done[ndesc]
    size_t counter_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    uint32_t ndesc = 0, nitems = 0;
    void drop() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (qmem) {
            cudaFree(qmem);
            account_device_bytes(-int64_t(qbytes));
        }
        qmem = nullptr;
        qbytes = 0;
        g_in = nullptr;
        g_out = nullptr;
    }
};

struct kfft_plan_uneven {
    uint32_t flags = 0;
    std::vector<uint32_t> lengths;
    std::vector<uint64_t> offsets;
    std::vector<size_t> ws_offsets;  // workspace slice of each sequence
    uint64_t total = 0;
    DeviceArena arena;
    std::map<uint32_t, std::unique_ptr<FftPlan>> plans;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    void* stage = nullptr;  // host staging: in and out, total points each
    UnevenQueue whole;                // the whole batch, for device buffers
    std::vector<UnevenQueue> groups;  // contiguous groups, for host buffers
    std::mutex mu;
    ~kfft_plan_uneven() {
        whole.drop();
        for (UnevenQueue& q : groups) q.drop();
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

// Builds the pass chain of every sequence of Q's range and the level-ordered
// queue of item records (each with the pass it waits for), uploads them and
// records the graph.
bool record(kfft_plan_uneven* P, UnevenQueue& Q, const vec2_t* in, vec2_t* out) {
    std::vector<PassDesc> all;
    std::vector<int32_t> deps;
    std::vector<uint32_t> level;
    char* base = static_cast<char*>(P->ws);
    for (size_t i = Q.s0; i < Q.s1; ++i) {
        const uint32_t n = P->lengths[i];
        if (n == 0) continue;
        const FftPlan& fp = *P->plans[n];
        Workspace ws;
        ws.base = base + P->ws_offsets[i];
        ws.size = workspace_bytes(fp, 1);
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
    for (PassDesc& d : all) {
        if (!d.regmode) return false;  // the queue kernel runs register-resident tiles only
        d.tc = 0;  // and its radix-16 stages on CUDA cores (a smaller kernel)
    }
    std::vector<Item> items;
    uint32_t smem = 0;
    for (uint32_t d = 0; d < nd; ++d) {
        smem = std::max(smem, all[d].smem_bytes);
        const int32_t dep = deps[d];
        const uint32_t need = dep >= 0 ? all[dep].tiles : 0u;
        for (uint32_t t = 0; t < all[d].tiles; ++t) items.push_back({d, t, dep, need});
    }
    // level order (dependencies first), larger tiles first within a level.
    // (Ordering groups of sequences in a diagonal wavefront instead, so that
    // a pass reads its predecessor's output from L2, measured slower: 10.6
    // against 10.1 ms on the default uneven batch with 2^21-point groups, and
    // 15-21 ms with smaller groups, from dependency waits.)
    std::stable_sort(items.begin(), items.end(), [&](const Item& a, const Item& b) {
        if (level[a.desc] != level[b.desc]) return level[a.desc] < level[b.desc];
        const uint64_t wa = uint64_t(all[a.desc].R) * all[a.desc].C;
        const uint64_t wb = uint64_t(all[b.desc].R) * all[b.desc].C;
        return wa > wb;
    });
    const size_t b_desc = a256(sizeof(PassDesc) * nd);
    const size_t b_extra = a256(pass_extra_bytes() * nd);
    const size_t b_item = a256(sizeof(Item) * items.size());
    const size_t b_cnt = a256(sizeof(uint32_t) * (nd + 2));
    Q.drop();
    Q.qbytes = b_desc + b_extra + b_item + b_cnt;
    if (cudaMalloc(&Q.qmem, Q.qbytes) != cudaSuccess) {
        cudaGetLastError();
        Q.qmem = nullptr;
        return false;
    }
    account_device_bytes(int64_t(Q.qbytes));
    char* q = static_cast<char*>(Q.qmem);
    PassDesc* d_desc = reinterpret_cast<PassDesc*>(q);
    void* d_extra = q + b_desc;
    Item* d_item = reinterpret_cast<Item*>(q + b_desc + b_extra);
    Q.counters = reinterpret_cast<uint32_t*>(q + b_desc + b_extra + b_item);
    Q.counter_bytes = sizeof(uint32_t) * (nd + 2);
    std::vector<char> extras(pass_extra_bytes() * nd);
    fill_extras(all.data(), extras.data(), nd);
    cudaStream_t st = cudaStreamPerThread;
    cudaMemcpyAsync(d_desc, all.data(), sizeof(PassDesc) * nd, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_extra, extras.data(), extras.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_item, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return false;
    Q.ndesc = nd;
    Q.nitems = uint32_t(items.size());

    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(Q.counters, 0, Q.counter_bytes, cap);
        if (Q.nitems)
            launch_persistent(d_desc, d_extra, d_item, Q.nitems, Q.counters,
                              Q.counters + 2, Q.counters + 1, smem, cap);
        e = cudaStreamEndCapture(cap, &graph);
    }
    if (Q.nitems) count_launch(-1);  // counted on every replay instead
    if (e == cudaSuccess) e = cudaGraphInstantiate(&Q.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        Q.exec = nullptr;
        return false;
    }
    Q.g_in = in;
    Q.g_out = out;
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

// copy streams of this host thread for the host-buffer path
struct CopyPair {
    cudaStream_t in = nullptr, out = nullptr;
};

CopyPair* copy_pair() {
    thread_local CopyPair cp;
    if (!cp.in) {
        if (cudaStreamCreateWithFlags(&cp.in, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&cp.out, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            cp.in = cp.out = nullptr;
            return nullptr;
        }
    }
    return &cp;
}

kfft_return_t launch(kfft_plan_uneven* P, UnevenQueue& Q, const vec2_t* in, vec2_t* out,
                     cudaStream_t st) {
    if (!Q.exec || Q.g_in != in || Q.g_out != out) {
        if (!record(P, Q, in, out)) return KFFT_RET_BUFFER_FAIL;
    }
    cudaError_t e = cudaGraphLaunch(Q.exec, st);
    count_graph_launch();
    if (Q.nitems) count_launch(1);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        return KFFT_RET_BUFFER_FAIL;
    }
    return KFFT_RET_SUCCESS;
}

// Contiguous groups of about equal points for the host-buffer path: copies
// of one group overlap the transform of its neighbours.
// Host-buffer calls split the batch into at most KFFT_UNEVEN_GROUPS groups
// of at least 2^KFFT_UNEVEN_GROUP_LOG2 points (measured on the default uneven
// batch with aligned copies: 12 groups 14.97 ms per e2e call, 16 14.62, 24
// 14.31, 32 14.35; before the copies were aligned 64 groups took 30.3 ms).
#ifndef KFFT_UNEVEN_GROUPS
#define KFFT_UNEVEN_GROUPS 24
#endif
#ifndef KFFT_UNEVEN_GROUP_LOG2
#define KFFT_UNEVEN_GROUP_LOG2 23
#endif
void make_groups(kfft_plan_uneven* P) {
    constexpr uint64_t kGroupPoints = uint64_t(1) << KFFT_UNEVEN_GROUP_LOG2;
    const size_t count = P->lengths.size();
    const uint64_t k = std::min<uint64_t>(KFFT_UNEVEN_GROUPS, P->total / kGroupPoints);
    if (k < 2 || count < 2) return;
    std::vector<std::pair<size_t, size_t>> ranges;
    size_t s = 0;
    for (uint64_t g = 0; g < k && s < count; ++g) {
        const size_t s0 = s;
        const uint64_t target = chunk_start(g + 1, k, P->total);
        if (g + 1 == k) s = count;
        while (s < count && (s == s0 || P->offsets[s] + P->lengths[s] <= target)) ++s;
        ranges.push_back({s0, s});
    }
    if (ranges.size() < 2 || ranges.back().second != count) return;
    P->groups.resize(ranges.size());
    for (size_t g = 0; g < ranges.size(); ++g) {
        UnevenQueue& Q = P->groups[g];
        Q.s0 = ranges[g].first;
        Q.s1 = ranges[g].second;
        Q.p0 = P->offsets[Q.s0];
        Q.p1 = Q.s1 < count ? P->offsets[Q.s1] : P->total;
    }
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
    P->ws_offsets.assign(count, 0);
    const int sign = (flags & KFFT_FLAG_INVERSE) ? +1 : -1;
    cudaStream_t st = cudaStreamPerThread;
    size_t ws = 0;
    for (uint32_t i = 0; i < count; ++i) {
        P->offsets[i] = P->total;
        P->total += lengths[i];
        const uint32_t n = lengths[i];
        if (n == 0) continue;
        if (!P->plans.count(n)) {
            // a tuned variant is used when it keeps every pass in register
            // tiles (the queue kernel's only tile kind); the record step checks
            const int tv = tuned_plan_variant(n, flags);
            PlanVariant var = tv >= 0 ? plan_variant(uint32_t(tv)) : PlanVariant();
            if (var.no_fused) var = PlanVariant();
            var.tile_cap = std::min<uint32_t>(var.tile_cap, KFFT_QUEUE_TILE);
            var.rmax = std::min<uint32_t>(var.rmax, KFFT_QUEUE_RMAX);
            FftPlan* fp = make_plan(n, sign, P->arena, st, kUnevenMaxPrime, var);
            if (!fp) return NULL;
            P->plans[n].reset(fp);
        }
        P->ws_offsets[i] = ws;
        ws += a256(workspace_bytes(*P->plans[n], 1));
    }
    P->whole.s0 = 0;
    P->whole.s1 = count;
    P->whole.p1 = P->total;
    make_groups(P.get());
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
    kfft_return_t r = launch(plan, plan->whole, reinterpret_cast<const vec2_t*>(fin),
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
    if (hin) din = s_in;
    if (hout) dout = s_out;
    std::vector<UnevenQueue*> used;
    CopyPair* cp = ((hin || hout) && !plan->groups.empty()) ? copy_pair() : nullptr;
    if (cp) {
        // group g's copy in, transform and copy out overlap its neighbours'
        std::vector<cudaEvent_t> evs;
        auto event = [&]() {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                return (cudaEvent_t) nullptr;
            }
            evs.push_back(e);
            return e;
        };
        kfft_return_t r = KFFT_RET_SUCCESS;
        for (size_t g = 0; g < plan->groups.size(); ++g) {
            UnevenQueue& Q = plan->groups[g];
            const CopyRange cr = copy_range(sizeof(vec2_t) * Q.p0, sizeof(vec2_t) * Q.p1, bytes,
                                            g == 0, g + 1 == plan->groups.size());
            if (hin) {
                cudaMemcpyAsync(reinterpret_cast<char*>(s_in) + cr.in0,
                                reinterpret_cast<const char*>(fin) + cr.in0, cr.in1 - cr.in0,
                                cudaMemcpyHostToDevice, cp->in);
                cudaEvent_t e = event();
                if (!e) {
                    r = KFFT_RET_BUFFER_FAIL;
                    break;
                }
                cudaEventRecord(e, cp->in);
                cudaStreamWaitEvent(st, e, 0);
            }
            r = launch(plan, Q, din, dout, st);
            if (r != KFFT_RET_SUCCESS) break;
            used.push_back(&Q);
            if (hout) {
                cudaEvent_t e = event();
                if (!e) {
                    r = KFFT_RET_BUFFER_FAIL;
                    break;
                }
                cudaEventRecord(e, st);
                cudaStreamWaitEvent(cp->out, e, 0);
                cudaMemcpyAsync(reinterpret_cast<char*>(fout) + cr.out0,
                                reinterpret_cast<const char*>(dout) + cr.out0, cr.out1 - cr.out0,
                                cudaMemcpyDeviceToHost, cp->out);
            }
        }
        if (hout) {
            cudaEvent_t e = event();
            if (e) {
                cudaEventRecord(e, cp->out);
                cudaStreamWaitEvent(st, e, 0);
            }
        }
        cudaError_t se = cudaStreamSynchronize(st);
        for (cudaEvent_t e : evs) cudaEventDestroy(e);
        if (se != cudaSuccess) note_cuda_error(se);
        if (r != KFFT_RET_SUCCESS) return r;
    } else {
        if (hin) cudaMemcpyAsync(s_in, fin, bytes, cudaMemcpyHostToDevice, st);
        kfft_return_t r = launch(plan, plan->whole, din, dout, st);
        if (r != KFFT_RET_SUCCESS) return r;
        used.push_back(&plan->whole);
        if (hout) cudaMemcpyAsync(fout, dout, bytes, cudaMemcpyDeviceToHost, st);
    }
    // the queue kernel's error word: set when a dependency wait gave up
    std::vector<uint32_t> words(used.size(), 0);
    for (size_t i = 0; i < used.size(); ++i)
        cudaMemcpyAsync(&words[i], used[i]->counters + 1, sizeof(uint32_t),
                        cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) note_cuda_error(e);
    uint32_t err = 0;
    for (uint32_t w : words) err |= w;
    if (take_pending_error() || err) return KFFT_RET_BUFFER_FAIL;
    return KFFT_RET_SUCCESS;
}

KFFT_API void kfft_release_uneven(kfft_plan_uneven* plan) { delete plan; }

// Failure-detection check of the queue kernel without a GPU fault: a queue of
// empty passes whose second item depends on the first.  With `satisfiable`
// 0 the first item is left out of the queue, so the dependency counter is a
// flag nothing sets: the wait gives up after max_polls polls, sets the error
// word and the kernel returns.  Returns the error word, or -1 on a CUDA error.
KFFT_API int kfft_gb300_queue_selftest(uint32_t max_polls, int satisfiable) {
    if (!ensure_device()) return -1;
    const size_t b_desc = a256(2 * sizeof(PassDesc));
    const size_t b_extra = a256(2 * pass_extra_bytes());
    const size_t b_item = a256(2 * sizeof(Item));
    const size_t b_cnt = a256(4 * sizeof(uint32_t));
    void* mem = nullptr;
    if (cudaMalloc(&mem, b_desc + b_extra + b_item + b_cnt) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    char* q = static_cast<char*>(mem);
    PassDesc d[2];
    memset(d, 0, sizeof(d));
    for (PassDesc& x : d) {  // a length-1 pass over zero sequences: no memory access
        x.tiles = 1;
        x.C = 1;
        x.lanes_j = 1;
        x.batch = 0;
        x.threads = kPassThreads;
    }
    const Item items[2] = {{0, 0, -1, 0}, {1, 0, 0, 1}};
    const Item* first = satisfiable ? items : items + 1;
    const uint32_t nitems = satisfiable ? 2u : 1u;
    std::vector<char> extras(2 * pass_extra_bytes(), 0);
    cudaStream_t st = cudaStreamPerThread;
    uint32_t* counters = reinterpret_cast<uint32_t*>(q + b_desc + b_extra + b_item);
    cudaMemcpyAsync(q, d, sizeof(d), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(q + b_desc, extras.data(), extras.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(q + b_desc + b_extra, first, nitems * sizeof(Item), cudaMemcpyHostToDevice,
                    st);
    cudaMemsetAsync(counters, 0, 4 * sizeof(uint32_t), st);
    launch_persistent(reinterpret_cast<PassDesc*>(q), q + b_desc, q + b_desc + b_extra, nitems,
                      counters, counters + 2, counters + 1, 0, st, max_polls);
    uint32_t err = 0;
    cudaMemcpyAsync(&err, counters + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(mem);
    if (e != cudaSuccess || take_pending_error()) {
        note_cuda_error(e);
        return -1;
    }
    return int(err);
}

}  // extern "C"
