// api.cu -- the C ABI of the GB300 FFT engine (drop-in for the reference kfft.h).
//
// Every exported function keeps the reference's name, argument meaning and
// error behaviour; the comment above each cites the reference definition it
// replaces.  Plans keep kfft_object_t as their first member (KFFT_PLAN_MMGR)
// and live in a kfft_pool_t exactly as the reference's do
// (KFFT_ALGO_PLAN_PREPARE, incs/kfft_algo.h:15-39): NULL pool and NULL lenmem
// creates a private pool, a non-NULL lenmem with NULL pool is a size query,
// a user pool receives the plan (KFFT_FLAG_RENEW clears it first).  The device
// side of each plan (its HBM arena of FP64-generated tables) is registered in
// the pool and freed with it.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.cuh"
#include "kfft.h"

using namespace kfft;

// ===========================================================================
// runtime state
// ===========================================================================
namespace kfft {
static std::atomic<uint64_t> g_launches{0};
static std::atomic<uint64_t> g_graphs{0};
static std::atomic<int64_t> g_bytes{0};
static std::atomic<int> g_last_err{0};
static std::mutex g_err_mu;
static std::string g_err_text;
static int g_device = -1;
static std::once_flag g_dev_once;

void count_launch(int64_t n) { g_launches += uint64_t(n); }
void count_graph_launch() { g_graphs += 1; }
void account_device_bytes(int64_t d) { g_bytes += d; }

static thread_local int t_pending = 0;

void note_cuda_error(cudaError_t e) {
    if (e == cudaSuccess) return;
    t_pending = int(e);
    g_last_err = int(e);
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err_text = cudaGetErrorString(e);
}

void note_engine_error(const char* msg) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err_text = msg;
}

bool ensure_device() {
    std::call_once(g_dev_once, [] {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            g_device = -1;
            std::lock_guard<std::mutex> lk(g_err_mu);
            g_err_text = "no CUDA device available";
            return;
        }
        int d = 0;
        cudaGetDevice(&d);
        g_device = d;
    });
    if (g_device < 0) return false;
    cudaSetDevice(g_device);
    return true;
}

int current_device() { return g_device; }

int take_pending_error() {
    int e = t_pending;
    t_pending = 0;
    return e;
}
}  // namespace kfft

// ===========================================================================
// device plan handle, placed in the plan's pool
// ===========================================================================
// One cached device workspace per host thread that evaluates the plan: the
// plan's tables are read-only, so evaluations of one plan from several host
// threads run concurrently, each on its own workspace and its own per-thread
// stream (the reference lets threads share a plan, ext/2d/kfft_cpx2.c:100-104).
struct WorkspaceSlot {
    std::thread::id owner;
    void* ws = nullptr;
    size_t size = 0;
};

struct kfft_gpu_plan {
    DeviceArena* arena = nullptr;
    FftPlan* plan = nullptr;      // complex transform (or the basis of a real plan)
    const vec2_t* super_tw = nullptr;  // real transform post/pre twiddles
    std::mutex* mu = nullptr;     // guards `slots` (held only to find a slot)
    std::deque<WorkspaceSlot>* slots = nullptr;  // a deque: slots never move
    void release() {
        if (slots) {
            for (WorkspaceSlot& s : *slots)
                if (s.ws) {
                    cudaFree(s.ws);
                    account_device_bytes(-int64_t(s.size));
                }
        }
        delete slots;
        slots = nullptr;
        delete plan;
        plan = nullptr;
        delete arena;
        arena = nullptr;
        delete mu;
        mu = nullptr;
    }
    // this host thread's device workspace of at least `bytes`, growing its
    // cached one (only the owning thread ever touches a slot's buffer)
    void* workspace(size_t bytes) {
        WorkspaceSlot* slot = nullptr;
        {
            std::lock_guard<std::mutex> lk(*mu);
            const std::thread::id me = std::this_thread::get_id();
            for (WorkspaceSlot& s : *slots)
                if (s.owner == me) slot = &s;
            if (!slot) {
                slots->push_back(WorkspaceSlot());
                slot = &slots->back();
                slot->owner = me;
            }
        }
        if (bytes <= slot->size) return slot->ws;
        if (slot->ws) {
            cudaFree(slot->ws);
            account_device_bytes(-int64_t(slot->size));
            slot->ws = nullptr;
            slot->size = 0;
        }
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            note_cuda_error(e);
            return nullptr;
        }
        slot->ws = p;
        slot->size = bytes;
        account_device_bytes(int64_t(bytes));
        return p;
    }
};

namespace kfft {
const FftPlan* device_plan_of(const kfft_plan_cpx* p) {
    return (p && p->gpu) ? p->gpu->plan : nullptr;
}
}  // namespace kfft

namespace {
struct PoolRegistry {
    std::vector<kfft_gpu_plan*> plans;
};

size_t gpu_handle_bytes() { return (sizeof(kfft_gpu_plan) + 15) & ~size_t(15); }

void registry_release(kfft_pool_t* A) {
    if (!A || !A->device) return;
    PoolRegistry* r = static_cast<PoolRegistry*>(A->device);
    for (kfft_gpu_plan* g : r->plans) g->release();
    r->plans.clear();
}

kfft_gpu_plan* new_gpu_handle(kfft_pool_t* A) {
    void* mem = kfft_pool_alloc(A, gpu_handle_bytes());
    if (!mem) return nullptr;
    kfft_gpu_plan* g = new (mem) kfft_gpu_plan();
    g->mu = new std::mutex();
    g->slots = new std::deque<WorkspaceSlot>();
    g->arena = new DeviceArena();
    if (!A->device) A->device = new PoolRegistry();
    static_cast<PoolRegistry*>(A->device)->plans.push_back(g);
    return g;
}

bool is_device_pointer(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Shared stream of synchronous evaluations on this host thread.
cudaStream_t sync_stream() { return cudaStreamPerThread; }

kfft_return_t finish(cudaStream_t st) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) note_cuda_error(e);
    const bool wait_failed = take_wait_failures(st);
    if (wait_failed) note_engine_error("a bounded bulk-copy wait ran out; the output is incomplete");
    const int pending = take_pending_error();
    return (pending || wait_failed) ? KFFT_RET_BUFFER_FAIL : KFFT_RET_SUCCESS;
}

real_t inverse_scale(uint32_t flags, uint32_t n) {
    if (!(flags & KFFT_FLAG_INVERSE) || (flags & KFFT_FLAG_DISABLE_NORM) || n == 0) return real_t(1);
    return real_t(1.0 / double(n));
}

// Staged view of a caller buffer on the device.
struct Staged {
    void* dev = nullptr;
    bool host = false;
};

// Workspace carved out of one device allocation: [staging | engine workspace].
struct Carve {
    char* base = nullptr;
    size_t used = 0, size = 0;
    void* take(size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        if (used + bytes > size) return nullptr;
        void* p = base + used;
        used += bytes;
        return p;
    }
};

size_t r256(size_t b) { return (b + 255) & ~size_t(255); }

// A convolution's spectrum product fused into the store of the last pass
// that writes a spectrum: with `mul` set (a spectrum in the same layout as the
// output), the last pass's plain store becomes out = v * mul, and *fused
// tells the caller that no separate product sweep is needed.  Passes whose
// last store already carries an element operation (Rader, Bluestein) keep it
// and leave *fused false.
struct Product {
    const vec2_t* mul = nullptr;
    bool* fused = nullptr;
};

void attach_product(std::vector<PassDesc>& descs, const Product& pr) {
    if (pr.fused) *pr.fused = false;
    if (!pr.mul || descs.empty() || descs.back().epi_op != EPI_NONE) return;
    descs.back().epi_op = EPI_MUL_OUT;
    descs.back().epi_tab = pr.mul;
    if (pr.fused) *pr.fused = true;
}

// Runs the complex transform of `g` on device buffers.
bool run_cpx(const FftPlan& P, const vec2_t* din, vec2_t* dout, uint32_t batch, real_t scale,
             void* wsmem, size_t wsbytes, cudaStream_t st, const Product& pr = Product()) {
    Workspace ws;
    ws.base = static_cast<char*>(wsmem);
    ws.size = wsbytes;
    Layout l;
    l.batch = batch;
    l.bs = P.N;
    std::vector<PassDesc> descs;
    if (!build_passes(P, din, l, dout, l, scale, ws, descs)) return false;
    attach_product(descs, pr);
    run_passes(descs, st);
    return true;
}

// Column transform of a (rows=y, cols=x) complex array in place; `pitch`
// (direct plans only; 0: x) is the row stride when only the first x columns
// of wider rows are transformed.
bool run_columns(const FftPlan& Py, vec2_t* data, uint32_t x, uint32_t y, real_t scale,
                 Carve& cv, cudaStream_t st, const Product& pr = Product(), uint32_t pitch = 0) {
    if (pr.fused) *pr.fused = false;
    if (pitch && pitch != x && Py.method != METHOD_DIRECT) return false;
    if (Py.method == METHOD_DIRECT) {
        Layout l;
        l.batch = x;
        l.bs = 1;
        l.es = pitch ? pitch : x;
        l.order = ORDER_B;
        size_t wb = workspace_bytes(Py, x);
        Workspace ws;
        ws.base = static_cast<char*>(cv.take(wb));
        ws.size = wb;
        if (wb && !ws.base) return false;
        std::vector<PassDesc> descs;
        if (!build_passes(Py, data, l, data, l, scale, ws, descs)) return false;
        attach_product(descs, pr);
        run_passes(descs, st);
        return true;
    }
    const size_t n = size_t(x) * y;
    vec2_t* t1 = static_cast<vec2_t*>(cv.take(n * sizeof(vec2_t)));
    vec2_t* t2 = static_cast<vec2_t*>(cv.take(n * sizeof(vec2_t)));
    size_t wb = workspace_bytes(Py, x);
    void* w = cv.take(wb);
    if (!t1 || !t2 || (wb && !w)) return false;
    launch_transpose(data, t1, y, x, 1, st);
    if (!run_cpx(Py, t1, t2, x, scale, w, wb, st)) return false;
    launch_transpose(t2, data, x, y, 1, st);
    return true;
}

size_t columns_bytes(const FftPlan& Py, uint32_t x, uint32_t y) {
    if (Py.method == METHOD_DIRECT) return r256(workspace_bytes(Py, x));
    return 2 * r256(sizeof(vec2_t) * size_t(x) * y) + r256(workspace_bytes(Py, x));
}

// Copy streams of this host thread for the chunked host-buffer path: copies
// in, compute and copies out of successive chunks overlap.
struct CopyStreams {
    cudaStream_t in = nullptr, out = nullptr;
};

CopyStreams* copy_streams() {
    thread_local CopyStreams cs;
    if (!cs.in) {
        if (cudaStreamCreateWithFlags(&cs.in, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&cs.out, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            cs.in = cs.out = nullptr;
            return nullptr;
        }
    }
    return &cs;
}

// Number of chunks a host-buffer batch of `bytes` in `batch` sequences is
// split into so that its copies overlap the transform (1: no split).
uint32_t host_chunks(size_t bytes, uint32_t batch) {
    constexpr size_t kChunkBytes = size_t(4) << 20;
    if (batch < 2 || bytes < 4 * kChunkBytes) return 1;
    size_t k = bytes / kChunkBytes;
    if (k > 16) k = 16;
    if (k > batch) k = batch;
    return uint32_t(k);
}

// Events of one chunked call (released when the call returns; the stream
// waits recorded on them have been enqueued by then).
struct EventSet {
    std::vector<cudaEvent_t> ev;
    cudaEvent_t get() {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        ev.push_back(e);
        return e;
    }
    ~EventSet() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
};

// A batched call whose input and/or output is in host memory, split into
// `chunks` ranges of sequences: chunk k's copy in, transform (`run(b0, b1)`
// on the compute stream `st`) and copy out run on three streams, so the
// copies of one chunk overlap the transforms of its neighbours.  in_per and
// out_per are bytes per sequence; h_in/h_out are the host buffers (null when
// that side is on the device) and d_in/d_out their device counterparts.
// The host buffers must not overlap.
template <class Run>
kfft_return_t chunked_host_call(uint32_t batch, uint32_t chunks, size_t in_per, size_t out_per,
                                const void* h_in, void* d_in, void* h_out, const void* d_out,
                                cudaStream_t st, Run run) {
    CopyStreams* cs = copy_streams();
    if (!cs) return KFFT_RET_BUFFER_FAIL;
    EventSet evs;
    const size_t tin = in_per * batch, tout = out_per * batch;
    for (uint32_t k = 0; k < chunks; ++k) {
        const uint32_t b0 = uint32_t(chunk_start(k, chunks, batch));
        const uint32_t b1 = uint32_t(chunk_start(k + 1, chunks, batch));
        const bool first = k == 0, last = k + 1 == chunks;
        if (h_in) {
            const CopyRange cr = copy_range(in_per * b0, in_per * b1, tin, first, last);
            cudaMemcpyAsync(static_cast<char*>(d_in) + cr.in0, static_cast<const char*>(h_in) + cr.in0,
                            cr.in1 - cr.in0, cudaMemcpyHostToDevice, cs->in);
            cudaEvent_t e = evs.get();
            if (!e) return KFFT_RET_BUFFER_FAIL;
            cudaEventRecord(e, cs->in);
            cudaStreamWaitEvent(st, e, 0);
        }
        if (!run(b0, b1)) return KFFT_RET_BUFFER_FAIL;
        if (h_out) {
            const CopyRange cr = copy_range(out_per * b0, out_per * b1, tout, first, last);
            cudaEvent_t e = evs.get();
            if (!e) return KFFT_RET_BUFFER_FAIL;
            cudaEventRecord(e, st);
            cudaStreamWaitEvent(cs->out, e, 0);
            cudaMemcpyAsync(static_cast<char*>(h_out) + cr.out0,
                            static_cast<const char*>(d_out) + cr.out0, cr.out1 - cr.out0,
                            cudaMemcpyDeviceToHost, cs->out);
        }
    }
    if (h_out) {
        cudaEvent_t e = evs.get();
        if (!e) return KFFT_RET_BUFFER_FAIL;
        cudaEventRecord(e, cs->out);
        cudaStreamWaitEvent(st, e, 0);
    }
    return finish(st);
}

bool ranges_overlap(const void* a, size_t na, const void* b, size_t nb) {
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + nb && y < x + na;
}

}  // namespace

// ===========================================================================
// pool (kfft_pool.c:33-96)
// ===========================================================================
extern "C" {

KFFT_API kfft_pool_t* kfft_pool_create(const size_t size) {
    const size_t memneed = sizeof(kfft_pool_t) + size;
    kfft_pool_t* p = static_cast<kfft_pool_t*>(malloc(memneed));
    if (!p) return NULL;
    memset(p, 0, sizeof(kfft_pool_t));
    p->allocated = memneed;
    p->align = 0;
    p->head = p->area;
    p->tail = p->area + size;
    p->cur = p->head;
    p->device = NULL;
    return p;
}

KFFT_API void* kfft_pool_alloc(kfft_pool_t* A, const size_t nmem) {
    static std::mutex mu;  // pool allocation is serialised (kfft_pool.c:57)
    if (!A || nmem == 0) return NULL;
    std::lock_guard<std::mutex> lk(mu);
    if (A->cur + nmem > A->tail) return NULL;
    uint8_t* r = A->cur;
    A->cur += nmem;
    return r;
}

KFFT_API size_t kfft_pool_empty(const kfft_pool_t* A) {
    return A ? size_t(A->tail - A->cur) : 0;
}

KFFT_API void kfft_pool_zmem(const kfft_pool_t* A, void* ptr, const size_t size) {
    if (A && ptr && size > 0 && static_cast<uint8_t*>(ptr) + size <= A->tail) memset(ptr, 0, size);
}

KFFT_API void kfft_pool_clear(kfft_pool_t* A) {
    if (!A) return;
    registry_release(A);
    kfft_pool_zmem(A, A->area, size_t(A->tail - A->head));
    A->cur = A->head;
}

KFFT_API void kfft_pool_free(kfft_pool_t* A) {
    if (!A) return;
    registry_release(A);
    delete static_cast<PoolRegistry*>(A->device);
    A->device = NULL;
    free(A);
}

}  // extern "C"

// ===========================================================================
// plan construction protocol (incs/kfft_algo.h:15-51)
// ===========================================================================
namespace {

template <typename T>
T* plan_prepare(uint32_t flags, size_t memneed, kfft_pool_t* A, size_t* lenmem,
                kfft_pool_t** owner) {
    T* plan = nullptr;
    kfft_pool_t* mm = nullptr;
    if (lenmem == NULL) {
        mm = A ? A : kfft_pool_create(memneed);
        if (mm) {
            if (A && (flags & KFFT_FLAG_RENEW)) kfft_pool_clear(mm);
            plan = static_cast<T*>(kfft_pool_alloc(mm, sizeof(T)));
        }
        if (!plan && !A) kfft_pool_free(mm);
    } else {
        if (A && *lenmem >= memneed) {
            mm = A;
            if (flags & KFFT_FLAG_RENEW) kfft_pool_clear(mm);
            plan = static_cast<T*>(kfft_pool_alloc(mm, sizeof(T)));
        }
        if (!plan) *lenmem = memneed;
    }
    if (plan) {
        memset(plan, 0, sizeof(T));
        plan->object.mmgr = mm;
    }
    *owner = mm;
    return plan;
}

template <typename T>
void plan_terminate(T* plan, kfft_pool_t* A) {
    if (A == NULL && plan) kfft_pool_free(plan->object.mmgr);
}

// host bytes of a complex plan in a pool
size_t cpx_memneed(uint32_t nfft) {
    return sizeof(kfft_plan_cpx) + (nfft ? gpu_handle_bytes() + 16 : 0);
}

// tuning table: (nfft, direction and tensor-core bits) -> plan variant
constexpr uint32_t kTuneKeyFlags = KFFT_FLAG_INVERSE | KFFT_FLAG_TENSOR_CORES;
std::mutex g_tune_mu;
std::unordered_map<uint64_t, uint32_t> g_tune;

uint64_t tune_key(uint32_t nfft, uint32_t flags) {
    return (uint64_t(nfft) << 32) | (flags & kTuneKeyFlags);
}

// the variant a plan built without an explicit choice uses, -1 if none
int tuned_variant(uint32_t nfft, uint32_t flags) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(nfft, flags));
    return it == g_tune.end() ? -1 : int(it->second);
}

bool variant_allowed(uint32_t variant, uint32_t flags) {
    if (variant >= kfft_variant_count()) return false;
    // the tensor-core variant only where the caller accepts its accuracy
    if (plan_variant(variant).tc && !(flags & KFFT_FLAG_TENSOR_CORES)) return false;
    return true;
}

// builds the device side of a complex plan node allocated in pool mm
bool cpx_init(kfft_plan_cpx* P, uint32_t nfft, uint32_t flags, kfft_pool_t* mm,
              int variant = -1) {
    P->nfft = nfft;
    P->flags = flags;
    P->level = 0;
    if (nfft == 0) return true;
    if (!ensure_device()) return false;
    kfft_gpu_plan* g = new_gpu_handle(mm);
    if (!g) return false;
    const int sign = (flags & KFFT_FLAG_INVERSE) ? +1 : -1;
    cudaStream_t st = sync_stream();
    // an explicit or tuned variant fixes every knob, tensor cores included;
    // otherwise the default split runs and the flag alone decides them
    const int chosen = variant >= 0 ? variant : tuned_variant(nfft, flags);
    uint32_t v = chosen >= 0 ? uint32_t(chosen) : 0u;
    if (!variant_allowed(v, flags)) v = 0;
    g->plan = make_plan(nfft, sign, *g->arena, st, kMaxDirectPrime, plan_variant(v));
    if (!g->plan) return false;
#if defined(KFFT_HALF_SCALAR)
    if (chosen < 0) set_tensor_cores(g->plan, (flags & KFFT_FLAG_TENSOR_CORES) != 0);
#endif
    if (finish(st) != KFFT_RET_SUCCESS) return false;
    P->gpu = g;
    const FftPlan& fp = *g->plan;
    P->method = fp.method;
    P->prm_count = fp.method == METHOD_DIRECT ? 0 : 1;
    const FftPlan& dp = fp.method == METHOD_DIRECT ? fp : *fp.sub_fwd;
    uint32_t rem = dp.N;
    P->fac_count = 0;
    for (size_t i = 0; i < dp.passes.size() && i < MAX_FACTORS; ++i) {
        rem /= dp.passes[i].R;
        P->factors[2 * i] = dp.passes[i].R;
        P->factors[2 * i + 1] = rem;
        P->fac_count++;
    }
    return true;
}

}  // namespace

namespace kfft {
// The tuned plan variant of (nfft, flags) for planners outside this file (the
// uneven batch), or -1 when none is recorded or it is not allowed.
int tuned_plan_variant(uint32_t nfft, uint32_t flags) {
    const int v = tuned_variant(nfft, flags);
    return (v >= 0 && variant_allowed(uint32_t(v), flags)) ? v : -1;
}
}  // namespace kfft

// ===========================================================================
// complex 1D (kfft_cpx.c:315-366)
// ===========================================================================
extern "C" {

KFFT_API kfft_plan_cpx* kfft_config_cpx(const uint32_t nfft, const uint32_t flags, kfft_pool_t* A,
                                        size_t* lenmem) {
    kfft_pool_t* mm = nullptr;
    kfft_plan_cpx* P = plan_prepare<kfft_plan_cpx>(flags, cpx_memneed(nfft), A, lenmem, &mm);
    if (!P) return NULL;
    if (!cpx_init(P, nfft, flags, mm)) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

KFFT_API uint32_t kfft_variant_count(void) {
#if defined(KFFT_HALF_SCALAR)
    return kPlanVariants;
#else
    return kPlanVariants - 1;  // no tensor-core variant in the double build
#endif
}

KFFT_API kfft_plan_cpx* kfft_config_cpx_variant(uint32_t nfft, uint32_t flags, uint32_t variant,
                                                kfft_pool_t* A, size_t* lenmem) {
    if (!variant_allowed(variant, flags)) return NULL;
    kfft_pool_t* mm = nullptr;
    kfft_plan_cpx* P = plan_prepare<kfft_plan_cpx>(flags, cpx_memneed(nfft), A, lenmem, &mm);
    if (!P) return NULL;
    if (!cpx_init(P, nfft, flags, mm, int(variant))) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

KFFT_API kfft_return_t kfft_tune_set(uint32_t nfft, uint32_t flags, uint32_t variant) {
    if (nfft == 0 || !variant_allowed(variant, flags)) return KFFT_RET_BADARGUMENTS;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_key(nfft, flags)] = variant;
    return KFFT_RET_SUCCESS;
}

KFFT_API int kfft_tune_get(uint32_t nfft, uint32_t flags) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(nfft, flags));
    return it == g_tune.end() ? -1 : int(it->second);
}

KFFT_API void kfft_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

KFFT_API kfft_return_t kfft_eval_cpx_batch(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                           kfft_cpx* fout, uint32_t batch) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0 || batch == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->gpu;
    if (!g || !g->plan) return KFFT_RET_IMPROPER_PLAN;
    cudaSetDevice(current_device());
    cudaStream_t st = sync_stream();
    const FftPlan& P = *g->plan;
    const size_t bytes = sizeof(vec2_t) * size_t(P.N) * batch;
    const bool hin = !is_device_pointer(fin), hout = !is_device_pointer(fout);
    const size_t wsb = workspace_bytes(P, batch);
    size_t need = r256(wsb) + (hin ? r256(bytes) : 0) + (hout ? r256(bytes) : 0);
    Carve cv;
    cv.base = static_cast<char*>(g->workspace(need));
    cv.size = need;
    if (need && !cv.base) return KFFT_RET_BUFFER_FAIL;
    const vec2_t* din = reinterpret_cast<const vec2_t*>(fin);
    vec2_t* dout = reinterpret_cast<vec2_t*>(fout);
    vec2_t* stage_in = nullptr;
    if (hin) {
        stage_in = static_cast<vec2_t*>(cv.take(bytes));
        din = stage_in;
    }
    if (hout) dout = (hin && fin == fout) ? stage_in : static_cast<vec2_t*>(cv.take(bytes));
    void* w = cv.take(wsb);
    const real_t scale = inverse_scale(plan->flags, plan->nfft);
    const uint32_t chunks = (hin || hout) ? host_chunks(bytes, batch) : 1;
    CopyStreams* cs = chunks > 1 ? copy_streams() : nullptr;
    if (cs) {
        // chunk k's copy in, transform and copy out overlap the neighbouring
        // chunks' (sequences are independent; the workspace serves one chunk
        // at a time on the compute stream)
        EventSet evs;
        const size_t per = sizeof(vec2_t) * size_t(P.N);
        for (uint32_t k = 0; k < chunks; ++k) {
            const uint32_t b0 = uint32_t(chunk_start(k, chunks, batch));
            const uint32_t b1 = uint32_t(chunk_start(k + 1, chunks, batch));
            const size_t off = size_t(b0) * P.N;
            const CopyRange cr = copy_range(per * b0, per * b1, bytes, k == 0, k + 1 == chunks);
            if (hin) {
                cudaMemcpyAsync(reinterpret_cast<char*>(stage_in) + cr.in0,
                                reinterpret_cast<const char*>(fin) + cr.in0, cr.in1 - cr.in0,
                                cudaMemcpyHostToDevice, cs->in);
                cudaEvent_t e = evs.get();
                if (!e) return KFFT_RET_BUFFER_FAIL;
                cudaEventRecord(e, cs->in);
                cudaStreamWaitEvent(st, e, 0);
            }
            if (!run_cpx(P, din + off, dout + off, b1 - b0, scale, w, wsb, st))
                return KFFT_RET_BUFFER_FAIL;
            if (hout) {
                cudaEvent_t e = evs.get();
                if (!e) return KFFT_RET_BUFFER_FAIL;
                cudaEventRecord(e, st);
                cudaStreamWaitEvent(cs->out, e, 0);
                cudaMemcpyAsync(reinterpret_cast<char*>(fout) + cr.out0,
                                reinterpret_cast<const char*>(dout) + cr.out0, cr.out1 - cr.out0,
                                cudaMemcpyDeviceToHost, cs->out);
            }
        }
        if (hout) {
            cudaEvent_t e = evs.get();
            if (!e) return KFFT_RET_BUFFER_FAIL;
            cudaEventRecord(e, cs->out);
            cudaStreamWaitEvent(st, e, 0);
        }
        return finish(st);
    }
    if (hin) cudaMemcpyAsync(stage_in, fin, bytes, cudaMemcpyHostToDevice, st);
    if (!run_cpx(P, din, dout, batch, scale, w, wsb, st)) return KFFT_RET_BUFFER_FAIL;
    if (hout) cudaMemcpyAsync(fout, dout, bytes, cudaMemcpyDeviceToHost, st);
    return finish(st);
}

KFFT_API kfft_return_t kfft_eval_cpx(kfft_plan_cpx* plan, const kfft_cpx* fin, kfft_cpx* fout) {
    return kfft_eval_cpx_batch(plan, fin, fout, 1);
}

KFFT_API kfft_return_t kfft_eval_cpx_async(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                           kfft_cpx* fout, uint32_t batch, void* stream) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0 || batch == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->gpu;
    if (!g || !g->plan) return KFFT_RET_IMPROPER_PLAN;
    cudaSetDevice(current_device());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const FftPlan& P = *g->plan;
    const size_t wsb = workspace_bytes(P, batch);
    void* w = wsb ? g->workspace(wsb) : nullptr;
    if (wsb && !w) return KFFT_RET_BUFFER_FAIL;
    if (!run_cpx(P, reinterpret_cast<const vec2_t*>(fin), reinterpret_cast<vec2_t*>(fout), batch,
                 inverse_scale(plan->flags, plan->nfft), w, wsb, st))
        return KFFT_RET_BUFFER_FAIL;
    return take_pending_error() ? KFFT_RET_BUFFER_FAIL : KFFT_RET_SUCCESS;
}

// ===========================================================================
// real ("scalar") 1D (kfft_scalar.c:295-329)
// ===========================================================================
KFFT_API kfft_plan_sclr* kfft_config_scalar(const uint32_t nfft, const uint32_t flags,
                                            kfft_pool_t* A, size_t* lenmem) {
    const uint32_t basis_n = (nfft % 2) ? nfft : nfft / 2;
    const size_t memneed = sizeof(kfft_plan_sclr) + cpx_memneed(basis_n) + gpu_handle_bytes() + 16;
    kfft_pool_t* mm = nullptr;
    kfft_plan_sclr* P = plan_prepare<kfft_plan_sclr>(flags, memneed, A, lenmem, &mm);
    if (!P) return NULL;
    P->nfft = nfft;
    P->flags = flags;
    P->basis = static_cast<kfft_plan_cpx*>(kfft_pool_alloc(mm, sizeof(kfft_plan_cpx)));
    if (!P->basis) {
        plan_terminate(P, A);
        return NULL;
    }
    memset(P->basis, 0, sizeof(kfft_plan_cpx));
    P->basis->object.mmgr = mm;
    if (!cpx_init(P->basis, basis_n, KFFT_CHECK_FLAGS(flags), mm)) {
        plan_terminate(P, A);
        return NULL;
    }
    if (nfft % 2 == 0 && nfft > 0) {
        kfft_gpu_plan* g = new_gpu_handle(mm);
        if (!g) {
            plan_terminate(P, A);
            return NULL;
        }
        const uint32_t h = nfft / 2;
        vec2_t* t = static_cast<vec2_t*>(g->arena->alloc(sizeof(vec2_t) * (h ? h : 1)));
        if (!t) {
            plan_terminate(P, A);
            return NULL;
        }
        gen_super_twiddles(t, h, (flags & KFFT_FLAG_INVERSE) ? +1 : -1, sync_stream());
        if (finish(sync_stream()) != KFFT_RET_SUCCESS) {
            plan_terminate(P, A);
            return NULL;
        }
        g->super_tw = t;
        P->gpu = g;
    }
    return P;
}

namespace {
uint32_t real_bins(const kfft_plan_sclr* p) {
    const uint32_t n = p->nfft;
    if (n % 2 || (p->flags & KFFT_FLAG_EXPAND_SCALAR)) return n;
    return n / 2 + 1;
}

// forward real transform on device buffers; spectrum stride `bins`
bool real_forward_dev(const kfft_plan_sclr* p, const real_t* din, vec2_t* dout, uint32_t batch,
                      uint64_t out_bs, int expand, Carve& cv, cudaStream_t st,
                      const Product& pr = Product()) {
    if (pr.fused) *pr.fused = false;
    const uint32_t n = p->nfft;
    const FftPlan& B = *p->basis->gpu->plan;
    if (n % 2) {
        vec2_t* w = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * size_t(n) * batch));
        size_t wb = workspace_bytes(B, batch);
        void* ws = cv.take(wb);
        if (!w || (wb && !ws)) return false;
        launch_widen(din, w, uint64_t(n) * batch, st);
        Workspace wsp;
        wsp.base = static_cast<char*>(ws);
        wsp.size = wb;
        Layout li;
        li.batch = batch;
        li.bs = n;
        Layout lo = li;
        lo.bs = out_bs;
        std::vector<PassDesc> d;
        if (!build_passes(B, w, li, dout, lo, real_t(1), wsp, d)) return false;
        attach_product(d, pr);
        run_passes(d, st);
        return true;
    }
    const uint32_t h = n / 2;
    vec2_t* z = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * size_t(h) * batch));
    size_t wb = workspace_bytes(B, batch);
    void* ws = cv.take(wb);
    if (!z || (wb && !ws)) return false;
    if (!run_cpx(B, reinterpret_cast<const vec2_t*>(din), z, batch, real_t(1), ws, wb, st))
        return false;
    launch_real_post(z, dout, p->gpu->super_tw, h, batch, out_bs, expand, st, pr.mul);
    if (pr.fused && pr.mul) *pr.fused = true;
    return true;
}

size_t real_forward_bytes(const kfft_plan_sclr* p, uint32_t batch) {
    const uint32_t n = p->nfft;
    const FftPlan& B = *p->basis->gpu->plan;
    const uint32_t m = (n % 2) ? n : n / 2;
    return r256(sizeof(vec2_t) * size_t(m) * batch) + r256(workspace_bytes(B, batch));
}

// inverse real transform on device buffers; spectrum stride in_bs
bool real_inverse_dev(const kfft_plan_sclr* p, const vec2_t* din, uint64_t in_bs, real_t* dout,
                      uint32_t batch, Carve& cv, cudaStream_t st) {
    const uint32_t n = p->nfft;
    const FftPlan& B = *p->basis->gpu->plan;
    if (n % 2) {
        vec2_t* w = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * size_t(n) * batch));
        size_t wb = workspace_bytes(B, batch);
        void* ws = cv.take(wb);
        if (!w || (wb && !ws)) return false;
        Workspace wsp;
        wsp.base = static_cast<char*>(ws);
        wsp.size = wb;
        Layout li;
        li.batch = batch;
        li.bs = in_bs;
        Layout lo = li;
        lo.bs = n;
        std::vector<PassDesc> d;
        if (!build_passes(B, din, li, w, lo, inverse_scale(p->flags, n), wsp, d)) return false;
        run_passes(d, st);
        launch_narrow(w, dout, uint64_t(n) * batch, st);
        return true;
    }
    const uint32_t h = n / 2;
    vec2_t* z = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * size_t(h) * batch));
    size_t wb = workspace_bytes(B, batch);
    void* ws = cv.take(wb);
    if (!z || (wb && !ws)) return false;
    launch_real_pre(din, z, p->gpu->super_tw, h, batch, in_bs, st);
    // the N/2-point basis normalises by 2/N: the reference's even-N inverse returns 2*x
    return run_cpx(B, z, reinterpret_cast<vec2_t*>(dout), batch, inverse_scale(p->flags, h), ws, wb,
                   st);
}

size_t real_inverse_bytes(const kfft_plan_sclr* p, uint32_t batch) {
    return real_forward_bytes(p, batch);
}
}  // namespace

KFFT_API kfft_return_t kfft_eval_scalar_batch(kfft_plan_sclr* plan, const kfft_scalar* fin,
                                              kfft_cpx* fout, uint32_t batch) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (!plan->basis || (plan->basis->flags & KFFT_FLAG_INVERSE)) return KFFT_RET_IMPROPER_PLAN;
    if (plan->nfft == 0 || batch == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->basis->gpu;
    cudaSetDevice(current_device());
    cudaStream_t st = sync_stream();
    const uint32_t bins = real_bins(plan);
    const size_t ib = sizeof(real_t) * size_t(plan->nfft) * batch;
    const size_t ob = sizeof(vec2_t) * size_t(bins) * batch;
    const bool hin = !is_device_pointer(fin), hout = !is_device_pointer(fout);
    size_t need = real_forward_bytes(plan, batch) + (hin ? r256(ib) : 0) + (hout ? r256(ob) : 0);
    Carve cv;
    cv.base = static_cast<char*>(g->workspace(need));
    cv.size = need;
    if (need && !cv.base) return KFFT_RET_BUFFER_FAIL;  // nothing to carve: no buffer needed
    const real_t* din = reinterpret_cast<const real_t*>(fin);
    vec2_t* dout = reinterpret_cast<vec2_t*>(fout);
    const int expand = (plan->flags & KFFT_FLAG_EXPAND_SCALAR) ? 1 : 0;
    const uint32_t chunks = ((hin || hout) && !(hin && hout && ranges_overlap(fin, ib, fout, ob)))
                                ? host_chunks(std::max(ib, ob), batch) : 1;
    if (chunks > 1) {
        // staging for the host sides, then scratch for the largest chunk
        if (hin) din = static_cast<const real_t*>(cv.take(ib));
        if (hout) dout = static_cast<vec2_t*>(cv.take(ob));
        Carve scratch = cv;
        const size_t n = plan->nfft;
        return chunked_host_call(batch, chunks, sizeof(real_t) * n, sizeof(vec2_t) * bins,
                                 hin ? fin : nullptr, const_cast<real_t*>(din),
                                 hout ? fout : nullptr, dout, st, [&](uint32_t b0, uint32_t b1) {
                                     Carve c = scratch;  // chunks run one after another on st
                                     return real_forward_dev(plan, din + n * b0, dout + size_t(bins) * b0,
                                                             b1 - b0, bins, expand, c, st);
                                 });
    }
    if (hin) {
        void* s = cv.take(ib);
        cudaMemcpyAsync(s, fin, ib, cudaMemcpyHostToDevice, st);
        din = static_cast<const real_t*>(s);
    }
    if (hout) dout = static_cast<vec2_t*>(cv.take(ob));
    if (!real_forward_dev(plan, din, dout, batch, bins, expand, cv, st))
        return KFFT_RET_BUFFER_FAIL;
    if (hout) cudaMemcpyAsync(fout, dout, ob, cudaMemcpyDeviceToHost, st);
    return finish(st);
}

KFFT_API kfft_return_t kfft_eval_scalar(kfft_plan_sclr* plan, const kfft_scalar* fin,
                                        kfft_cpx* fout) {
    return kfft_eval_scalar_batch(plan, fin, fout, 1);
}

KFFT_API kfft_return_t kfft_evali_scalar_batch(kfft_plan_sclr* plan, const kfft_cpx* fin,
                                               kfft_scalar* fout, uint32_t batch) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (!plan->basis || !(plan->basis->flags & KFFT_FLAG_INVERSE)) return KFFT_RET_IMPROPER_PLAN;
    if (plan->nfft == 0 || batch == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->basis->gpu;
    cudaSetDevice(current_device());
    cudaStream_t st = sync_stream();
    const uint32_t bins = real_bins(plan);
    const size_t ib = sizeof(vec2_t) * size_t(bins) * batch;
    const size_t ob = sizeof(real_t) * size_t(plan->nfft) * batch;
    const bool hin = !is_device_pointer(fin), hout = !is_device_pointer(fout);
    size_t need = real_inverse_bytes(plan, batch) + (hin ? r256(ib) : 0) + (hout ? r256(ob) : 0);
    Carve cv;
    cv.base = static_cast<char*>(g->workspace(need));
    cv.size = need;
    if (need && !cv.base) return KFFT_RET_BUFFER_FAIL;  // nothing to carve: no buffer needed
    const vec2_t* din = reinterpret_cast<const vec2_t*>(fin);
    real_t* dout = reinterpret_cast<real_t*>(fout);
    const uint32_t chunks = ((hin || hout) && !(hin && hout && ranges_overlap(fin, ib, fout, ob)))
                                ? host_chunks(std::max(ib, ob), batch) : 1;
    if (chunks > 1) {
        if (hin) din = static_cast<const vec2_t*>(cv.take(ib));
        if (hout) dout = static_cast<real_t*>(cv.take(ob));
        Carve scratch = cv;
        const size_t n = plan->nfft;
        return chunked_host_call(batch, chunks, sizeof(vec2_t) * bins, sizeof(real_t) * n,
                                 hin ? fin : nullptr, const_cast<vec2_t*>(din),
                                 hout ? fout : nullptr, dout, st, [&](uint32_t b0, uint32_t b1) {
                                     Carve c = scratch;  // chunks run one after another on st
                                     return real_inverse_dev(plan, din + size_t(bins) * b0, bins,
                                                             dout + n * b0, b1 - b0, c, st);
                                 });
    }
    if (hin) {
        void* s = cv.take(ib);
        cudaMemcpyAsync(s, fin, ib, cudaMemcpyHostToDevice, st);
        din = static_cast<const vec2_t*>(s);
    }
    if (hout) dout = static_cast<real_t*>(cv.take(ob));
    if (!real_inverse_dev(plan, din, bins, dout, batch, cv, st)) return KFFT_RET_BUFFER_FAIL;
    if (hout) cudaMemcpyAsync(fout, dout, ob, cudaMemcpyDeviceToHost, st);
    return finish(st);
}

KFFT_API kfft_return_t kfft_evali_scalar(kfft_plan_sclr* plan, const kfft_cpx* fin,
                                         kfft_scalar* fout) {
    return kfft_evali_scalar_batch(plan, fin, fout, 1);
}

// ===========================================================================
// service API (kfft_ext.c:6-95)
// ===========================================================================
KFFT_API void kfft_info(kfft_info_t* info) {
    if (!info) return;
    info->vmajor = KFFT_MAJOR_VERSION;
    info->vminor = KFFT_MINOR_VERSION;
    info->vpatch = KFFT_PATCH_VERSION;
    info->flags = KFFT_INFO_USE_SYSMATH | KFFT_INFO_RADER_ALGO;
#if defined(KFFT_HALF_SCALAR)
    info->flags |= KFFT_INFO_HALF_SCALAR;
#endif
}

KFFT_API uint32_t kfft_next_fast_size(uint32_t n) {
    while (1) {
        uint32_t m = n;
        while ((m % 2) == 0) m /= 2;
        while ((m % 3) == 0) m /= 3;
        while ((m % 5) == 0) m /= 5;
        if (m <= 1) break;
        n++;
    }
    return n;
}

KFFT_API void* kfft_malloc(uint32_t sz) {
    void* p = nullptr;
    if (posix_memalign(&p, 64, sz ? sz : 1) != 0) return NULL;
    return p;
}

KFFT_API void kfft_free_null(void** mem) {
    if (!mem) return;
    free(*mem);
    *mem = NULL;
}

KFFT_API kfft_return_t kfft_cleanup(void* mem) {
    if (!mem) return KFFT_RET_FREE_NULL;
    kfft_object_t* M = static_cast<kfft_object_t*>(mem);
    if (M->mmgr == NULL) return KFFT_RET_FREE_NULL;
    kfft_pool_free(M->mmgr);
    return KFFT_RET_SUCCESS;
}

static const char* kErrors[] = {"Success operation result",
                                "Internal allocation memory fail",
                                "Temporary buffer allocation fail",
                                "Invalide free() operation for NULL buffer",
                                "Use improper real function for this plan",
                                "Use missing argument for configure plan"};

KFFT_API const char* kfft_strerr(const kfft_return_t code) {
    if (code >= sizeof(kErrors) / sizeof(kErrors[0])) return "Unknown return code";
    return kErrors[code];
}

KFFT_API void kfft_gb300_stats(kfft_gb300_stats_t* s) {
    if (!s) return;
    s->kernel_launches = g_launches.load();
    s->graph_launches = g_graphs.load();
    s->device_bytes = uint64_t(g_bytes.load());
    s->device = g_device;
    s->last_cuda_error = g_last_err.load();
}

KFFT_API const char* kfft_gb300_last_error(void) {
    static thread_local std::string copy;
    std::lock_guard<std::mutex> lk(g_err_mu);
    copy = g_err_text;
    return copy.c_str();
}

KFFT_API const char* kfft_gb300_describe(const kfft_plan_cpx* plan) {
    static thread_local std::string s;
    if (!plan || !plan->gpu || !plan->gpu->plan) s = "";
    else s = describe(*plan->gpu->plan);
    return s.c_str();
}

}  // extern "C"

// ===========================================================================
// 2D complex and real (ext/2d/kfft_cpx2.c, ext/2d/kfft_scalar2.c)
// ===========================================================================
namespace {
const FftPlan* gp(const kfft_plan_cpx* p) { return p && p->gpu ? p->gpu->plan : nullptr; }
}  // namespace

extern "C" {

KFFT_API kfft_plan_c2d* kfft_config2_cpx(const uint32_t x_size, const uint32_t y_size,
                                         const uint32_t flags, kfft_pool_t* A, size_t* lenmem) {
    size_t memneed = sizeof(kfft_plan_c2d) + cpx_memneed(x_size) +
                     (x_size != y_size ? cpx_memneed(y_size) : 0) + 16;
    kfft_pool_t* mm = nullptr;
    kfft_plan_c2d* P = plan_prepare<kfft_plan_c2d>(flags, memneed, A, lenmem, &mm);
    if (!P) return NULL;
    P->nfft = x_size * y_size;
    P->x = x_size;
    P->y = y_size;
    P->flags = flags;
    const uint32_t cf = KFFT_CHECK_FLAGS(flags);
    P->plan_x = kfft_config_cpx(x_size, cf, mm, NULL);
    P->plan_y = (x_size == y_size) ? P->plan_x : kfft_config_cpx(y_size, cf, mm, NULL);
    if (!P->plan_x || !P->plan_y) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

}  // extern "C"

namespace {
// 2D complex transform on device buffers (rows of x, y rows)
bool c2d_dev(const kfft_plan_c2d* p, const vec2_t* din, vec2_t* dout, Carve& cv, cudaStream_t st,
             const Product& pr = Product()) {
    const FftPlan* Px = gp(p->plan_x);
    const FftPlan* Py = gp(p->plan_y);
    if (!Px || !Py) return false;
    const uint32_t x = p->x, y = p->y;
    size_t wb = workspace_bytes(*Px, y);
    void* w = cv.take(wb);
    if (wb && !w) return false;
    if (!run_cpx(*Px, din, dout, y, inverse_scale(p->flags, x), w, wb, st)) return false;
    return run_columns(*Py, dout, x, y, inverse_scale(p->flags, y), cv, st, pr);
}

size_t c2d_bytes(const kfft_plan_c2d* p) {
    return r256(workspace_bytes(*gp(p->plan_x), p->y)) + columns_bytes(*gp(p->plan_y), p->x, p->y);
}

// A 2D complex transform from host memory to host memory whose copy in
// overlaps the row passes: the rows arrive in chunks, each chunk's row
// transforms starting as soon as its copy lands.  The column passes need
// every row, and the copy out (one contiguous copy) waits for them.
// (Copying column blocks out by pitched copies under the next
// block's column passes measured slower: 14.1 against 11.6 ms per forward +
// inverse step of 8192^2 FP32, the single staged call 12.2 ms.)
constexpr uint32_t k2dRowChunks = 8;

bool c2d_pipelines(const kfft_plan_c2d* p, const void* fin, const void* fout) {
    const size_t bytes = sizeof(vec2_t) * size_t(p->x) * p->y;
    return bytes >= (size_t(16) << 20) && p->y >= k2dRowChunks && !is_device_pointer(fin) &&
           !is_device_pointer(fout);
}

kfft_return_t c2d_host_pipelined(const kfft_plan_c2d* p, const vec2_t* fin, vec2_t* fout,
                                 kfft_gpu_plan* g) {
    cudaSetDevice(current_device());
    cudaStream_t st = sync_stream();
    CopyStreams* cs = copy_streams();
    if (!cs) return KFFT_RET_BUFFER_FAIL;
    const FftPlan& Px = *gp(p->plan_x);
    const FftPlan& Py = *gp(p->plan_y);
    const uint32_t x = p->x, y = p->y;
    const size_t row_bytes = sizeof(vec2_t) * size_t(x);
    uint32_t max_rows = 0;
    for (uint32_t k = 0; k < k2dRowChunks; ++k)
        max_rows = std::max<uint32_t>(max_rows, uint32_t(chunk_start(k + 1, k2dRowChunks, y) -
                                                         chunk_start(k, k2dRowChunks, y)));
    const size_t wrow = workspace_bytes(Px, max_rows);
    const size_t need = r256(row_bytes * y) + r256(wrow) + columns_bytes(Py, x, y);
    Carve cv;
    cv.base = static_cast<char*>(g->workspace(need));
    cv.size = need;
    if (!cv.base) return KFFT_RET_BUFFER_FAIL;
    vec2_t* d = static_cast<vec2_t*>(cv.take(row_bytes * y));
    void* wr = cv.take(wrow);
    EventSet evs;
    for (uint32_t k = 0; k < k2dRowChunks; ++k) {
        const uint32_t r0 = uint32_t(chunk_start(k, k2dRowChunks, y));
        const uint32_t r1 = uint32_t(chunk_start(k + 1, k2dRowChunks, y));
        if (r1 <= r0) continue;
        cudaMemcpyAsync(d + size_t(r0) * x, fin + size_t(r0) * x, row_bytes * (r1 - r0),
                        cudaMemcpyHostToDevice, cs->in);
        cudaEvent_t e = evs.get();
        if (!e) return KFFT_RET_BUFFER_FAIL;
        cudaEventRecord(e, cs->in);
        cudaStreamWaitEvent(st, e, 0);
        if (!run_cpx(Px, d + size_t(r0) * x, d + size_t(r0) * x, r1 - r0, inverse_scale(p->flags, x),
                     wr, wrow, st))
            return KFFT_RET_BUFFER_FAIL;
    }
    if (!run_columns(Py, d, x, y, inverse_scale(p->flags, y), cv, st)) return KFFT_RET_BUFFER_FAIL;
    cudaMemcpyAsync(fout, d, row_bytes * y, cudaMemcpyDeviceToHost, st);
    return finish(st);
}

template <typename F>
kfft_return_t with_staging(kfft_gpu_plan* g, size_t work, const void* const* ins,
                           const size_t* in_bytes, int nin, void* out, size_t out_bytes, F&& body) {
    cudaSetDevice(current_device());
    cudaStream_t st = sync_stream();
    bool hin[4] = {false, false, false, false};
    size_t need = r256(work);
    for (int i = 0; i < nin; ++i) {
        hin[i] = !is_device_pointer(ins[i]);
        if (hin[i]) need += r256(in_bytes[i]);
    }
    const bool hout = !is_device_pointer(out);
    if (hout) need += r256(out_bytes);
    Carve cv;
    cv.base = static_cast<char*>(g->workspace(need));
    cv.size = need;
    if (need && !cv.base) return KFFT_RET_BUFFER_FAIL;  // nothing to carve: no buffer needed
    const void* dins[4];
    for (int i = 0; i < nin; ++i) {
        if (hin[i]) {
            void* s = cv.take(in_bytes[i]);
            cudaMemcpyAsync(s, ins[i], in_bytes[i], cudaMemcpyHostToDevice, st);
            dins[i] = s;
        } else {
            dins[i] = ins[i];
        }
    }
    void* dout = hout ? cv.take(out_bytes) : out;
    if (!body(dins, dout, cv, st)) return KFFT_RET_BUFFER_FAIL;
    if (hout) cudaMemcpyAsync(out, dout, out_bytes, cudaMemcpyDeviceToHost, st);
    return finish(st);
}
}  // namespace

extern "C" {

KFFT_API kfft_return_t kfft_eval2_cpx(kfft_plan_c2d* cfg, const kfft_cpx* fin, kfft_cpx* fout) {
    if (!cfg || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (cfg->nfft == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = cfg->plan_x->gpu;
    const size_t bytes = sizeof(vec2_t) * size_t(cfg->nfft);
    if (c2d_pipelines(cfg, fin, fout))
        return c2d_host_pipelined(cfg, reinterpret_cast<const vec2_t*>(fin),
                                  reinterpret_cast<vec2_t*>(fout), g);
    const void* ins[1] = {fin};
    return with_staging(g, c2d_bytes(cfg), ins, &bytes, 1, fout, bytes,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            return c2d_dev(cfg, static_cast<const vec2_t*>(di[0]),
                                           static_cast<vec2_t*>(dout), cv, st);
                        });
}

KFFT_API kfft_plan_s2d* kfft_config2_scalar(const uint32_t x_size, const uint32_t y_size,
                                            const uint32_t flags, kfft_pool_t* A, size_t* lenmem) {
    size_t rx = 0, ry = 0;
    const uint32_t cf = KFFT_CHECK_FLAGS(flags);
    // forward: real rows (expanded) + complex columns; inverse: complex rows + real columns
    if (flags & KFFT_FLAG_INVERSE) {
        rx = cpx_memneed(x_size);
        ry = sizeof(kfft_plan_sclr) + cpx_memneed(y_size) + 2 * gpu_handle_bytes() + 32;
    } else {
        rx = sizeof(kfft_plan_sclr) + cpx_memneed(x_size) + 2 * gpu_handle_bytes() + 32;
        ry = cpx_memneed(y_size);
    }
    size_t memneed = sizeof(kfft_plan_s2d) + rx + ry + 16;
    kfft_pool_t* mm = nullptr;
    kfft_plan_s2d* P = plan_prepare<kfft_plan_s2d>(flags, memneed, A, lenmem, &mm);
    if (!P) return NULL;
    P->nfft = x_size * y_size;
    P->x = x_size;
    P->y = y_size;
    P->flags = flags;
    if (flags & KFFT_FLAG_INVERSE) {
        P->plan_x = reinterpret_cast<kfft_object_t*>(kfft_config_cpx(x_size, cf, mm, NULL));
        P->plan_y = reinterpret_cast<kfft_object_t*>(
            kfft_config_scalar(y_size, cf | KFFT_FLAG_EXPAND_SCALAR, mm, NULL));
    } else {
        P->plan_x = reinterpret_cast<kfft_object_t*>(
            kfft_config_scalar(x_size, cf | KFFT_FLAG_EXPAND_SCALAR, mm, NULL));
        P->plan_y = reinterpret_cast<kfft_object_t*>(kfft_config_cpx(y_size, cf, mm, NULL));
    }
    if (!P->plan_x || !P->plan_y) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

}  // extern "C"

namespace {
// 1: an even-x real 2D forward transforms the columns of bins 0..x/2 only
// and fills the rest by Hermitian symmetry
#ifndef KFFT_S2D_FWD_HALF
#define KFFT_S2D_FWD_HALF 1
#endif
// real 2D forward on device: rows real (expanded) -> complex columns.  For an
// even x with a direct column plan, the rows keep bins 0..x/2, the columns run
// over those x/2 + 1 only, and bins k2 > x/2 are filled from
// X[k1][k2] = conj(X[-k1][x - k2]), the values the reference's columns of
// conjugate-mirrored row bins come to.
bool s2d_forward_dev(const kfft_plan_s2d* p, const real_t* din, vec2_t* dout, Carve& cv,
                     cudaStream_t st, const Product& pr = Product()) {
    const kfft_plan_sclr* rx = reinterpret_cast<const kfft_plan_sclr*>(p->plan_x);
    const kfft_plan_cpx* cy = reinterpret_cast<const kfft_plan_cpx*>(p->plan_y);
    if (KFFT_S2D_FWD_HALF && !pr.mul && p->x % 2 == 0 && p->x >= 4 &&
        gp(cy)->method == METHOD_DIRECT) {
        const uint32_t hx = p->x / 2 + 1;
        if (pr.fused) *pr.fused = false;
        if (!real_forward_dev(rx, din, dout, p->y, p->x, 0, cv, st)) return false;
        if (!run_columns(*gp(cy), dout, hx, p->y, real_t(1), cv, st, Product(), p->x)) return false;
        launch_hermitian_fill(dout, p->x, p->y, st);
        return true;
    }
    if (!real_forward_dev(rx, din, dout, p->y, p->x, 1, cv, st)) return false;
    return run_columns(*gp(cy), dout, p->x, p->y, real_t(1), cv, st, pr);
}
size_t s2d_forward_bytes(const kfft_plan_s2d* p) {
    const kfft_plan_sclr* rx = reinterpret_cast<const kfft_plan_sclr*>(p->plan_x);
    const kfft_plan_cpx* cy = reinterpret_cast<const kfft_plan_cpx*>(p->plan_y);
    return real_forward_bytes(rx, p->y) + columns_bytes(*gp(cy), p->x, p->y);
}
// 1: an even-y real 2D inverse runs down the columns with no transposes
#ifndef KFFT_S2D_INV_COLUMNS
#define KFFT_S2D_INV_COLUMNS 1
#endif
// real 2D inverse on device: complex rows -> real columns (ext/2d/kfft_scalar2.c:185-246).
// For an even y the columns' real inverse reads rows 0..y/2 only, so only
// those rows are transformed, and the inverse runs down the columns in place
// of the reference's per-column copies: the pre-twiddle down the columns, the
// y/2-point complex inverse over the x columns, then each complex row m split
// into real rows 2m and 2m+1 (4160^2 FP32 0.340 to 0.310 ms, 4096 x 4097
// 0.873 to 0.606 ms).  An odd y, and a y/2-point plan whose column tiles
// would hold fewer than four columns (8192^2: one 4096-point pass, 1.012
// against 0.913 ms through the transposes), keep the transposes.
bool s2d_inverse_dev(const kfft_plan_s2d* p, const vec2_t* din, real_t* dout, Carve& cv,
                     cudaStream_t st) {
    const kfft_plan_cpx* cx = reinterpret_cast<const kfft_plan_cpx*>(p->plan_x);
    const kfft_plan_sclr* ry = reinterpret_cast<const kfft_plan_sclr*>(p->plan_y);
    const uint32_t x = p->x, y = p->y;
    const size_t n = size_t(x) * y;
    if (KFFT_S2D_INV_COLUMNS && y % 2 == 0 && columns_coalesce(*ry->basis->gpu->plan)) {
        const uint32_t h = y / 2;
        const FftPlan& B = *ry->basis->gpu->plan;
        vec2_t* rows = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * size_t(x) * (h + 1)));
        vec2_t* z = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * size_t(x) * h));
        const size_t wb = workspace_bytes(*gp(cx), h + 1);
        void* w = cv.take(wb);
        if (!rows || !z || (wb && !w)) return false;
        if (!run_cpx(*gp(cx), din, rows, h + 1, inverse_scale(cx->flags, x), w, wb, st)) return false;
        launch_real_pre_cols(rows, z, ry->gpu->super_tw, h, x, x, x, st);
        // the h-point basis normalises by 2/y: the reference's even-length real inverse returns 2*x
        if (!run_columns(B, z, x, h, inverse_scale(ry->flags, h), cv, st)) return false;
        launch_split_rows(z, dout, h, x, st);
        return true;
    }
    vec2_t* rows = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * n));
    vec2_t* cols = static_cast<vec2_t*>(cv.take(sizeof(vec2_t) * n));
    real_t* rcols = static_cast<real_t*>(cv.take(sizeof(real_t) * n));
    size_t wb = workspace_bytes(*gp(cx), y);
    void* w = cv.take(wb);
    if (!rows || !cols || !rcols || (wb && !w)) return false;
    if (!run_cpx(*gp(cx), din, rows, y, inverse_scale(cx->flags, x), w, wb, st)) return false;
    launch_transpose(rows, cols, y, x, 1, st);
    if (!real_inverse_dev(ry, cols, y, rcols, x, cv, st)) return false;
    launch_transpose_real(rcols, dout, x, y, st);
    return true;
}
size_t s2d_inverse_bytes(const kfft_plan_s2d* p) {
    const kfft_plan_cpx* cx = reinterpret_cast<const kfft_plan_cpx*>(p->plan_x);
    const kfft_plan_sclr* ry = reinterpret_cast<const kfft_plan_sclr*>(p->plan_y);
    const size_t n = size_t(p->x) * p->y;
    if (KFFT_S2D_INV_COLUMNS && p->y % 2 == 0 && columns_coalesce(*ry->basis->gpu->plan)) {
        const uint32_t h = p->y / 2;
        return r256(sizeof(vec2_t) * size_t(p->x) * (h + 1)) + r256(sizeof(vec2_t) * size_t(p->x) * h) +
               r256(workspace_bytes(*gp(cx), h + 1)) +
               columns_bytes(*ry->basis->gpu->plan, p->x, h);
    }
    return 2 * r256(sizeof(vec2_t) * n) + r256(sizeof(real_t) * n) +
           r256(workspace_bytes(*gp(cx), p->y)) + real_inverse_bytes(ry, p->x);
}
kfft_gpu_plan* s2d_handle(const kfft_plan_s2d* p) {
    if (p->flags & KFFT_FLAG_INVERSE)
        return reinterpret_cast<const kfft_plan_cpx*>(p->plan_x)->gpu;
    return reinterpret_cast<const kfft_plan_cpx*>(p->plan_y)->gpu;
}

// The real conv2d plan as built here: the reference's struct (the base, so
// the caller's kfft_plan_s2cnv* is this object) and, for an even x, the two
// plans of the half-spectrum inverse.
struct S2cnvPlan : kfft_plan_s2cnv {
    kfft_plan_cpx* cols_inv;   // y-point complex inverse over the x/2 + 1 columns
    kfft_plan_sclr* rows_inv;  // x-point real inverse of each row from x/2 + 1 bins
};

bool s2cnv_half_spectrum(uint32_t x, uint32_t y) { return x >= 2 && x % 2 == 0 && y >= 1; }

// Circular 2D convolution of two real y-by-x arrays through half spectra (x
// even).  The rows' real transforms keep bins 0..x/2 (hx = x/2 + 1 a row),
// the column transforms run over those hx columns only, the spectrum product
// is fused into the second operand's last column pass, and the inverse runs
// the complex columns, then each row's real inverse from its hx bins: about
// half the column work and half the spectrum traffic of the expanded spectra
// (ext/conv2d/kfft_scalar_conv.c computes full spectra).  The result is the
// same: the factor 2 of an even-length real inverse (kfft_scalar.c:218-242),
// which the reference picks up in its columns when y is even, comes from the
// rows here, so an odd y takes a factor 1/2 in the column scale.
kfft_return_t s2cnv_half_eval(const S2cnvPlan* Q, const kfft_scalar* fin_A,
                              const kfft_scalar* fin_B, kfft_scalar* fout) {
    const kfft_plan_s2cnv* plan = Q;
    const kfft_plan_sclr* rx = reinterpret_cast<const kfft_plan_sclr*>(plan->plan_fwd->plan_x);
    const kfft_plan_cpx* cy = reinterpret_cast<const kfft_plan_cpx*>(plan->plan_fwd->plan_y);
    const uint32_t x = plan->x, y = plan->y, hx = x / 2 + 1;
    const size_t nh = size_t(hx) * y;
    const size_t rb = sizeof(real_t) * size_t(plan->nfft), hb = sizeof(vec2_t) * nh;
    const size_t fwd_work = real_forward_bytes(rx, y) + columns_bytes(*gp(cy), hx, y);
    const size_t inv_work =
        columns_bytes(*gp(Q->cols_inv), hx, y) + real_inverse_bytes(Q->rows_inv, y);
    const size_t work = 2 * r256(hb) + std::max(fwd_work, inv_work);
    real_t cscale = inverse_scale(Q->cols_inv->flags, y);
    if ((y % 2) && !(Q->cols_inv->flags & KFFT_FLAG_DISABLE_NORM)) cscale *= real_t(0.5);
    const void* ins[2] = {fin_A, fin_B};
    const size_t ibs[2] = {rb, rb};
    return with_staging(cy->gpu, work, ins, ibs, 2, fout, rb,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            vec2_t* fa = static_cast<vec2_t*>(cv.take(hb));
                            vec2_t* fb = static_cast<vec2_t*>(cv.take(hb));
                            if (!fa || !fb) return false;
                            const size_t mark = cv.used;
                            const real_t* a = static_cast<const real_t*>(di[0]);
                            const real_t* b = static_cast<const real_t*>(di[1]);
                            if (!real_forward_dev(rx, a, fa, y, hx, 0, cv, st)) return false;
                            if (!run_columns(*gp(cy), fa, hx, y, real_t(1), cv, st)) return false;
                            cv.used = mark;
                            if (!real_forward_dev(rx, b, fb, y, hx, 0, cv, st)) return false;
                            bool fused = false;
                            Product pr;
                            pr.mul = fa;
                            pr.fused = &fused;
                            if (!run_columns(*gp(cy), fb, hx, y, real_t(1), cv, st, pr)) return false;
                            cv.used = mark;
                            if (!fused) launch_hadamard(fb, fa, nh, st);
                            if (!run_columns(*gp(Q->cols_inv), fb, hx, y, cscale, cv, st)) return false;
                            return real_inverse_dev(Q->rows_inv, fb, hx, static_cast<real_t*>(dout), y,
                                                    cv, st);
                        });
}
}  // namespace

extern "C" {

KFFT_API kfft_return_t kfft_eval2_scalar(kfft_plan_s2d* plan, const kfft_scalar* fin,
                                         kfft_cpx* fout) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->flags & KFFT_FLAG_INVERSE) return KFFT_RET_IMPROPER_PLAN;
    if (plan->nfft == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = s2d_handle(plan);
    const size_t ib = sizeof(real_t) * size_t(plan->nfft), ob = sizeof(vec2_t) * size_t(plan->nfft);
    const void* ins[1] = {fin};
    return with_staging(g, s2d_forward_bytes(plan), ins, &ib, 1, fout, ob,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            return s2d_forward_dev(plan, static_cast<const real_t*>(di[0]),
                                                   static_cast<vec2_t*>(dout), cv, st);
                        });
}

KFFT_API kfft_return_t kfft_evali2_scalar(kfft_plan_s2d* plan, const kfft_cpx* fin,
                                          kfft_scalar* fout) {
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (!(plan->flags & KFFT_FLAG_INVERSE)) return KFFT_RET_IMPROPER_PLAN;
    if (plan->nfft == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = s2d_handle(plan);
    const size_t ib = sizeof(vec2_t) * size_t(plan->nfft), ob = sizeof(real_t) * size_t(plan->nfft);
    const void* ins[1] = {fin};
    return with_staging(g, s2d_inverse_bytes(plan), ins, &ib, 1, fout, ob,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            return s2d_inverse_dev(plan, static_cast<const vec2_t*>(di[0]),
                                                   static_cast<real_t*>(dout), cv, st);
                        });
}

// ===========================================================================
// 1D convolution (ext/conv/kfft_cpx_conv.c, ext/conv/kfft_scalar_conv.c)
// ===========================================================================
KFFT_API kfft_plan_ccnv* kfft_config_conv_cpx(const uint32_t nfft, const uint32_t flags,
                                              kfft_pool_t* A, size_t* lenmem) {
    size_t memneed = sizeof(kfft_plan_ccnv) + 2 * cpx_memneed(nfft) + 16;
    kfft_pool_t* mm = nullptr;
    kfft_plan_ccnv* P = plan_prepare<kfft_plan_ccnv>(flags, memneed, A, lenmem, &mm);
    if (!P) return NULL;
    P->nfft = nfft;
    P->flags = flags;
    const uint32_t cf = KFFT_CHECK_FLAGS_CCNV(flags);
    P->plan_fwd = kfft_config_cpx(nfft, cf, mm, NULL);
    P->plan_inv = kfft_config_cpx(nfft, cf | KFFT_FLAG_INVERSE, mm, NULL);
    if (!P->plan_fwd || !P->plan_inv) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

KFFT_API kfft_return_t kfft_eval_conv_cpx(kfft_plan_ccnv* plan, const kfft_cpx* fin_A,
                                          const kfft_cpx* fin_B, kfft_cpx* fout) {
    if (!plan || !fin_A || !fin_B || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->plan_fwd->gpu;
    const FftPlan& F = *gp(plan->plan_fwd);
    const FftPlan& I = *gp(plan->plan_inv);
    const uint32_t n = plan->nfft;
    const size_t bytes = sizeof(vec2_t) * size_t(n);
    const size_t work = 2 * r256(bytes) + r256(std::max(workspace_bytes(F, 1), workspace_bytes(I, 1)));
    const void* ins[2] = {fin_A, fin_B};
    const size_t ibs[2] = {bytes, bytes};
    return with_staging(g, work, ins, ibs, 2, fout, bytes,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            vec2_t* fa = static_cast<vec2_t*>(cv.take(bytes));
                            vec2_t* fb = static_cast<vec2_t*>(cv.take(bytes));
                            size_t wb = std::max(workspace_bytes(F, 1), workspace_bytes(I, 1));
                            void* w = cv.take(wb);
                            if (!fa || !fb || (wb && !w)) return false;
                            if (!run_cpx(F, static_cast<const vec2_t*>(di[0]), fa, 1, real_t(1), w, wb, st))
                                return false;
                            // the spectrum product rides on B's last forward pass when it can
                            bool fused = false;
                            Product pr;
                            pr.mul = fa;
                            pr.fused = &fused;
                            if (!run_cpx(F, static_cast<const vec2_t*>(di[1]), fb, 1, real_t(1), w, wb, st, pr))
                                return false;
                            if (!fused) launch_hadamard(fb, fa, n, st);
                            return run_cpx(I, fb, static_cast<vec2_t*>(dout), 1,
                                           inverse_scale(plan->plan_inv->flags, n), w, wb, st);
                        });
}

KFFT_API kfft_plan_scnv* kfft_config_conv_scalar(const uint32_t nfft, const uint32_t flags,
                                                 kfft_pool_t* A, size_t* lenmem) {
    const uint32_t basis_n = (nfft % 2) ? nfft : nfft / 2;
    size_t one = sizeof(kfft_plan_sclr) + cpx_memneed(basis_n) + gpu_handle_bytes() + 16;
    size_t memneed = sizeof(kfft_plan_scnv) + 2 * one + 16;
    kfft_pool_t* mm = nullptr;
    kfft_plan_scnv* P = plan_prepare<kfft_plan_scnv>(flags, memneed, A, lenmem, &mm);
    if (!P) return NULL;
    P->nfft = nfft;
    P->flags = flags;
    const uint32_t cf = KFFT_CHECK_FLAGS_CCNV(flags);
    P->plan_fwd = kfft_config_scalar(nfft, cf, mm, NULL);
    P->plan_inv = kfft_config_scalar(nfft, cf | KFFT_FLAG_INVERSE, mm, NULL);
    if (!P->plan_fwd || !P->plan_inv) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

KFFT_API kfft_return_t kfft_eval_conv_scalar(kfft_plan_scnv* plan, const kfft_scalar* fin_A,
                                             const kfft_scalar* fin_B, kfft_scalar* fout) {
    if (!plan || !fin_A || !fin_B || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->plan_fwd->basis->gpu;
    const uint32_t n = plan->nfft;
    const uint32_t bins = real_bins(plan->plan_fwd);
    const size_t rb = sizeof(real_t) * size_t(n);
    const size_t sb = sizeof(vec2_t) * size_t(bins);
    const size_t work = 2 * r256(sb) + real_forward_bytes(plan->plan_fwd, 1) +
                        real_inverse_bytes(plan->plan_inv, 1);
    const void* ins[2] = {fin_A, fin_B};
    const size_t ibs[2] = {rb, rb};
    return with_staging(g, work, ins, ibs, 2, fout, rb,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            vec2_t* fa = static_cast<vec2_t*>(cv.take(sb));
                            vec2_t* fb = static_cast<vec2_t*>(cv.take(sb));
                            if (!fa || !fb) return false;
                            int ex = (plan->plan_fwd->flags & KFFT_FLAG_EXPAND_SCALAR) ? 1 : 0;
                            size_t mark = cv.used;
                            if (!real_forward_dev(plan->plan_fwd, static_cast<const real_t*>(di[0]),
                                                  fa, 1, bins, ex, cv, st))
                                return false;
                            cv.used = mark;
                            bool fused = false;
                            Product pr;
                            pr.mul = fa;
                            pr.fused = &fused;
                            if (!real_forward_dev(plan->plan_fwd, static_cast<const real_t*>(di[1]),
                                                  fb, 1, bins, ex, cv, st, pr))
                                return false;
                            cv.used = mark;
                            if (!fused) launch_hadamard(fb, fa, bins, st);
                            return real_inverse_dev(plan->plan_inv, fb, bins,
                                                    static_cast<real_t*>(dout), 1, cv, st);
                        });
}

// ===========================================================================
// 2D convolution (ext/conv2d/kfft_cpx_conv.c, ext/conv2d/kfft_scalar_conv.c)
// ===========================================================================
KFFT_API kfft_plan_c2cnv* kfft_config2_conv_cpx(const uint32_t x, const uint32_t y,
                                                const uint32_t flags, kfft_pool_t* A,
                                                size_t* lenmem) {
    size_t one = sizeof(kfft_plan_c2d) + cpx_memneed(x) + (x != y ? cpx_memneed(y) : 0) + 16;
    size_t memneed = sizeof(kfft_plan_c2cnv) + 2 * one + 16;
    kfft_pool_t* mm = nullptr;
    kfft_plan_c2cnv* P = plan_prepare<kfft_plan_c2cnv>(flags, memneed, A, lenmem, &mm);
    if (!P) return NULL;
    P->nfft = x * y;
    P->x = x;
    P->y = y;  // the reference stores x here (ext/conv2d/kfft_cpx_conv.c:67); y is intended
    P->flags = flags;
    const uint32_t cf = KFFT_CHECK_FLAGS_CCNV(flags);
    P->plan_fwd = kfft_config2_cpx(x, y, cf, mm, NULL);
    P->plan_inv = kfft_config2_cpx(x, y, cf | KFFT_FLAG_INVERSE, mm, NULL);
    if (!P->plan_fwd || !P->plan_inv) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

KFFT_API kfft_return_t kfft_eval2_conv_cpx(kfft_plan_c2cnv* plan, const kfft_cpx* fin_A,
                                           const kfft_cpx* fin_B, kfft_cpx* fout) {
    if (!plan || !fin_A || !fin_B || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0) return KFFT_RET_SUCCESS;
    kfft_gpu_plan* g = plan->plan_fwd->plan_x->gpu;
    const size_t bytes = sizeof(vec2_t) * size_t(plan->nfft);
    const size_t work = 2 * r256(bytes) + std::max(c2d_bytes(plan->plan_fwd), c2d_bytes(plan->plan_inv));
    const void* ins[2] = {fin_A, fin_B};
    const size_t ibs[2] = {bytes, bytes};
    return with_staging(g, work, ins, ibs, 2, fout, bytes,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            vec2_t* fa = static_cast<vec2_t*>(cv.take(bytes));
                            vec2_t* fb = static_cast<vec2_t*>(cv.take(bytes));
                            if (!fa || !fb) return false;
                            size_t mark = cv.used;
                            if (!c2d_dev(plan->plan_fwd, static_cast<const vec2_t*>(di[0]), fa, cv, st))
                                return false;
                            cv.used = mark;
                            bool fused = false;
                            Product pr;
                            pr.mul = fa;
                            pr.fused = &fused;
                            if (!c2d_dev(plan->plan_fwd, static_cast<const vec2_t*>(di[1]), fb, cv, st, pr))
                                return false;
                            cv.used = mark;
                            if (!fused) launch_hadamard(fb, fa, plan->nfft, st);
                            return c2d_dev(plan->plan_inv, fb, static_cast<vec2_t*>(dout), cv, st);
                        });
}

KFFT_API kfft_plan_s2cnv* kfft_config2_conv_scalar(const uint32_t x, const uint32_t y,
                                                   const uint32_t flags, kfft_pool_t* A,
                                                   size_t* lenmem) {
    const uint32_t cf = KFFT_CHECK_FLAGS_CCNV(flags);
    size_t fwd = 0, inv = 0, cinv = 0, rinv = 0;
    kfft_config2_scalar(x, y, cf, NULL, &fwd);
    kfft_config2_scalar(x, y, cf | KFFT_FLAG_INVERSE, NULL, &inv);
    const bool half = s2cnv_half_spectrum(x, y);
    if (half) {
        kfft_config_cpx(y, cf | KFFT_FLAG_INVERSE, NULL, &cinv);
        kfft_config_scalar(x, cf | KFFT_FLAG_INVERSE, NULL, &rinv);
    }
    size_t memneed = sizeof(S2cnvPlan) + fwd + inv + cinv + rinv + 32;
    kfft_pool_t* mm = nullptr;
    S2cnvPlan* Q = plan_prepare<S2cnvPlan>(flags, memneed, A, lenmem, &mm);
    if (!Q) return NULL;
    kfft_plan_s2cnv* P = Q;
    P->nfft = x * y;
    P->x = x;
    P->y = y;
    P->flags = flags;
    P->plan_fwd = kfft_config2_scalar(x, y, cf, mm, NULL);
    P->plan_inv = kfft_config2_scalar(x, y, cf | KFFT_FLAG_INVERSE, mm, NULL);
    bool ok = P->plan_fwd && P->plan_inv;
    if (ok && half) {
        Q->cols_inv = kfft_config_cpx(y, cf | KFFT_FLAG_INVERSE, mm, NULL);
        Q->rows_inv = kfft_config_scalar(x, cf | KFFT_FLAG_INVERSE, mm, NULL);
        ok = Q->cols_inv && Q->rows_inv;
    }
    if (!ok) {
        plan_terminate(P, A);
        return NULL;
    }
    return P;
}

KFFT_API kfft_return_t kfft_eval2_conv_scalar(kfft_plan_s2cnv* plan, const kfft_scalar* fin_A,
                                              const kfft_scalar* fin_B, kfft_scalar* fout) {
    if (!plan || !fin_A || !fin_B || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0) return KFFT_RET_SUCCESS;
    const S2cnvPlan* Q = static_cast<const S2cnvPlan*>(plan);
    if (Q->cols_inv && Q->rows_inv) return s2cnv_half_eval(Q, fin_A, fin_B, fout);
    kfft_gpu_plan* g = s2d_handle(plan->plan_fwd);
    const size_t n = plan->nfft;
    const size_t rb = sizeof(real_t) * n, sb = sizeof(vec2_t) * n;
    const size_t work = 2 * r256(sb) + std::max(s2d_forward_bytes(plan->plan_fwd),
                                                s2d_inverse_bytes(plan->plan_inv));
    const void* ins[2] = {fin_A, fin_B};
    const size_t ibs[2] = {rb, rb};
    return with_staging(g, work, ins, ibs, 2, fout, rb,
                        [&](const void* const* di, void* dout, Carve& cv, cudaStream_t st) {
                            vec2_t* fa = static_cast<vec2_t*>(cv.take(sb));
                            vec2_t* fb = static_cast<vec2_t*>(cv.take(sb));
                            if (!fa || !fb) return false;
                            size_t mark = cv.used;
                            if (!s2d_forward_dev(plan->plan_fwd, static_cast<const real_t*>(di[0]), fa, cv, st))
                                return false;
                            cv.used = mark;
                            bool fused = false;
                            Product pr;
                            pr.mul = fa;
                            pr.fused = &fused;
                            if (!s2d_forward_dev(plan->plan_fwd, static_cast<const real_t*>(di[1]), fb, cv, st, pr))
                                return false;
                            cv.used = mark;
                            if (!fused) launch_hadamard(fb, fa, n, st);
                            return s2d_inverse_dev(plan->plan_inv, fb, static_cast<real_t*>(dout), cv, st);
                        });
}

}  // extern "C"
