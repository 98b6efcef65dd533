// engine.cuh -- internal interfaces of the GB300 FFT engine.
//
// A transform of length N is executed as a list of PassDesc records.  Each
// pass is one Stockham step of radix R (R = a sub-FFT length that fits in one
// CTA's shared memory) over a tile of C "lanes"; inside the CTA the length-R
// sub-FFT itself runs as Stockham passes of small radices (2..16 and odd
// primes up to 31) in shared memory.  Prime lengths become (p-1)-point cyclic
// convolutions (Rader) or M-point chirp convolutions (Bluestein); both are
// expressed as DIRECT sub-plans whose first/last passes carry fused
// prologue/epilogue element operations, so every kernel launch of the engine
// is one PassDesc (plus a few small elementwise kernels for the real
// transform's post-twiddle and for transposes).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <stdint.h>

#include <cstddef>
#include <string>
#include <vector>

#include "kfft.h"

namespace kfft {

#if defined(KFFT_HALF_SCALAR)
typedef float real_t;
typedef float2 vec2_t;
#else
typedef double real_t;
typedef double2 vec2_t;
#endif

// Largest radix handled inside a CTA by a dedicated butterfly.
constexpr int kMaxInnerRadices = 12;
// CTA size ceiling of the pass kernels (their register budget is sized for it).
constexpr uint32_t kPassThreads = 256;
// Largest tile (lanes x length) of the fused-I/O kernel (radices <= 16):
// the first inner pass reads global memory, the last writes it, and the
// passes between exchange through two shared-memory buffers.
constexpr uint32_t kRegTile = 4096;
// Largest prime factor a DIRECT plan accepts; larger primes go to Rader/Bluestein.
constexpr uint32_t kMaxDirectPrime = 31;

// ---- magic-number unsigned division, valid for every 32-bit numerator -----
struct FastDiv {
    uint32_t d;   // divisor
    uint32_t m;   // magic multiplier
    uint32_t s;   // shift
    void init(uint32_t div);
};

enum : uint8_t { MODE_LANE = 0, MODE_ELEM = 1 };
enum : uint8_t { ORDER_J = 0, ORDER_B = 1 };

// Prologue: how a pass obtains input element n of sequence b.
enum : uint8_t {
    PRO_NONE = 0,   // in[b*bs + n*es]
    PRO_CHIRP = 1,  // n < bound ? in[b*bs + n*es] * tab[n] : 0  (Bluestein pre-chirp + pad)
    PRO_GATHER = 2, // in[b*bs + perm[n]*es]                    (Rader generator gather)
};
// Epilogue: how a pass stores output element k of sequence b.
enum : uint8_t {
    EPI_NONE = 0,      // out[b*bs + k*es] = v * scale
    EPI_MUL = 1,       // out[b*bs + k*es] = v * tab[k]
    EPI_CHIRP = 2,     // k < bound: out[b*bs + k*es] = v * tab[k] * scale
    EPI_RADER_FWD = 3, // out[..k..] = v * tab[k]; k == 0: aux_out[2b] = x0, aux_out[2b+1] = x0 + v
    EPI_RADER_INV = 4, // aux_out[b*bs + perm[k]*es] = (v + x0) * scale; k == 0 also X_0
    EPI_MUL_OUT = 5,   // out[i] = v * tab[i] * scale, i = b*bs + k*es: a table in the output's
                       // layout (the other operand's spectrum of a convolution)
};

struct PassDesc {
    const vec2_t* in;
    vec2_t* out;
    uint64_t in_bs, out_bs;  // batch strides (elements)
    uint32_t in_es, out_es;  // element strides
    uint32_t batch;          // sequences
    uint32_t N;              // transform length at this level
    uint32_t R;              // sub-FFT length of this pass
    uint32_t Ns;             // product of the lengths of the previous passes
    uint32_t C;              // lanes per tile
    uint32_t lanes_j;        // N / R
    uint32_t tiles;          // ceil(batch * lanes_j / C)
    uint32_t threads;        // CTA size
    uint32_t smem_bytes;     // dynamic shared memory
    uint32_t lane_stride;    // compile-time bodies: shared-memory slots from one lane to the next
    uint8_t load_mode, store_mode, order;
    uint8_t inv;             // butterfly direction (tables already carry it)
    uint8_t regmode;         // fused-I/O tile (radices <= 16, C*R <= kRegTile)
    uint8_t tc;              // radix-16 inner passes on tensor cores (FP32 build)
    uint8_t nrad;
    uint8_t rad[kMaxInnerRadices];
    uint8_t spec;            // log2 R of a compile-time power-of-two tile body, 0: generic
    FastDiv div_R, div_lanes_j, div_batch, div_Ns, div_C;
    const vec2_t* tw_inner;  // W_R^i, i < R
    const vec2_t* tw_lo;     // W_N^i, i < 2^tw_shift
    const vec2_t* tw_hi;     // W_N^(i << tw_shift)
    uint32_t tw_shift;
    uint32_t tw_mul;         // N / (Ns * R) = lanes_j / Ns
    // fused element operations
    uint8_t pro_op, epi_op;
    const vec2_t* pro_tab;
    const uint32_t* pro_perm;
    uint32_t pro_bound;
    const vec2_t* epi_tab;
    const uint32_t* epi_perm;
    uint32_t epi_bound;
    const vec2_t* aux_in;   // Rader: the original input (x0)
    vec2_t* aux_out;        // Rader: the final output
    uint64_t aux_in_bs, aux_out_bs;
    uint32_t aux_out_es;
    real_t scale;
};

// ---- device tables -----------------------------------------------------
// Fills t[i] = exp(sign * 2 pi i * (i * mult mod n) / n) in FP64 for i < count.
void gen_twiddles(vec2_t* t, uint32_t count, uint64_t mult, uint32_t n, int sign,
                  cudaStream_t st);
// Bluestein chirp c[k] = exp(sign * i pi (k^2 mod 2n) / n), k < count.
void gen_chirp(vec2_t* c, uint32_t count, uint32_t n, int sign, cudaStream_t st);
// Bluestein filter b[m] = conj(c[|m|]) on the circle of m_len points (zero elsewhere).
void gen_bluestein_filter(vec2_t* b, const vec2_t* chirp, uint32_t n, uint32_t m_len,
                          cudaStream_t st);
// Rader: s[j] = W_p^(pidx[j]) for j < p-1.
void gen_rader_kernel(vec2_t* s, const uint32_t* pidx, uint32_t p, int sign, cudaStream_t st);
// Real-transform post-twiddle table st[k] = exp(sign * i pi ((k+1)/h + 1/2)), k < h.
void gen_super_twiddles(vec2_t* t, uint32_t h, int sign, cudaStream_t st);
// Scale a table in place: t[i] *= s.
void scale_table(vec2_t* t, uint32_t count, double s, cudaStream_t st);

// ---- kernels run by the executor ------------------------------------------
void launch_pass(const PassDesc& d, cudaStream_t st);
// Persistent work-queue execution of many pass chains in one launch: `items`
// lists 16-byte (desc, tile, dep, need) records ordered by dependency level;
// a tile of pass desc starts once done[dep] reaches need, the tile count of
// pass dep (dep -1: no dependency).  A bounded wait that gives up sets *error
// instead of hanging.  Every pass must be a register-resident tile
// (PassDesc::regmode).
size_t pass_extra_bytes();
void fill_extras(const PassDesc* d, void* extras, size_t n);
// A dependency wait polls at most max_polls times (about 200 ns apart) before
// it sets the error word and skips the tile; the default allows about 3 s.
constexpr uint32_t kQueueMaxPolls = 1u << 24;
bool launch_persistent(const PassDesc* descs, const void* extras,
                       const void* items, uint32_t nitems, uint32_t* head, uint32_t* done,
                       uint32_t* error, uint32_t smem_bytes, cudaStream_t st,
                       uint32_t max_polls = kQueueMaxPolls);
// Even-N real transform post-processing (kfft_scalar.c:174-216): z holds the
// N/2-point spectrum of each sequence, out gets nbins bins per sequence.
// With `mul` (a spectrum in the output's layout) every bin written is also
// multiplied by mul's bin: the product of a convolution, fused into the store.
void launch_real_post(const vec2_t* z, vec2_t* out, const vec2_t* st_tab, uint32_t h,
                      uint32_t batch, uint64_t out_bs, int expand, cudaStream_t st,
                      const vec2_t* mul = nullptr);
// Even-N real inverse pre-processing (kfft_scalar.c:218-242).
void launch_real_pre(const vec2_t* in, vec2_t* z, const vec2_t* st_tab, uint32_t h,
                     uint32_t batch, uint64_t in_bs, cudaStream_t st);
// The same down the `ncols` columns of row-major arrays (row strides in_rs,
// z_rs), and the split of the h complex rows it leads to into 2h real rows.
void launch_real_pre_cols(const vec2_t* in, vec2_t* z, const vec2_t* st_tab, uint32_t h,
                          uint32_t ncols, uint64_t in_rs, uint64_t z_rs, cudaStream_t st);
void launch_split_rows(const vec2_t* z, real_t* out, uint32_t h, uint32_t ncols, cudaStream_t st);
// Bins x/2+1 .. x-1 of a y-by-x 2D spectrum of real data from bins 0..x/2
// (x even, in place).
void launch_hermitian_fill(vec2_t* data, uint32_t x, uint32_t y, cudaStream_t st);
// Odd-N helpers: real -> complex widening and complex -> real narrowing with scale.
void launch_widen(const real_t* in, vec2_t* out, uint64_t n, cudaStream_t st);
void launch_narrow(const vec2_t* in, real_t* out, uint64_t n, cudaStream_t st);
// Batched out-of-place transpose of (rows x cols) matrices of complex / real.
void launch_transpose(const vec2_t* in, vec2_t* out, uint32_t rows, uint32_t cols,
                      uint32_t batch, cudaStream_t st);
void launch_transpose_real(const real_t* in, real_t* out, uint32_t rows, uint32_t cols,
                           cudaStream_t st);
// b[i] *= a[i] (complex), i < n -- the Hadamard product of the convolutions.
void launch_hadamard(vec2_t* b, const vec2_t* a, uint64_t n, cudaStream_t st);
// Generic strided copy used for compaction (rows of `len` out of stride `src_stride`).
void launch_copy_rows(const vec2_t* in, vec2_t* out, uint32_t len, uint64_t src_stride,
                      uint64_t dst_stride, uint32_t rows, cudaStream_t st);

// ---- host-side plan --------------------------------------------------------
enum Method : uint32_t { METHOD_DIRECT = 0, METHOD_RADER = 1, METHOD_BLUESTEIN = 2 };

struct PassSpec {
    uint32_t R, Ns;
    std::vector<uint8_t> radices;
    const vec2_t* tw_inner;
};

struct DeviceArena;  // device memory owned by a plan tree

// Planner knobs one plan variant fixes (the tuner's search space).
// Largest pass length of variant 0's multi-pass splits (a build-time knob for
// sweeps; variants 1 and 2 lower it to 512 and 256).
#ifndef KFFT_PLAN_RMAX
#define KFFT_PLAN_RMAX 1024
#endif
struct PlanVariant {
    uint32_t rmax = KFFT_PLAN_RMAX;  // largest pass length of a multi-pass split
    uint32_t lanes = 0;          // lanes of multi-pass tiles (0: precision default)
    uint32_t lanes_mul = 1;      // multiplier on the default lanes of multi-pass tiles
    uint32_t single_div = 1;     // divisor on the default lanes of single-pass tiles
    uint32_t single_cap = 4096;  // longest length run as one fused pass
    uint32_t tile_cap = kRegTile;  // most points per register tile
    bool reverse = false;        // multi-pass splits run longest pass last
    bool no_rader = false;       // primes through Bluestein even where Rader applies
    bool no_fused = false;       // shared-memory ping-pong tiles only
    bool tc = false;             // radix-16 stages on tensor cores (FP32 build)
};
// Variants 0..kPlanVariants-1; the tensor-core variant is always the last.
constexpr uint32_t kPlanVariants = 10;
PlanVariant plan_variant(uint32_t index);
// the variant the tuning table records for (nfft, flags), -1 if none
int tuned_plan_variant(uint32_t nfft, uint32_t flags);

struct FftPlan {
    uint32_t N = 0;
    PlanVariant var;
    int sign = -1;  // -1 forward, +1 inverse
    bool tc = false;  // radix-16 passes on tensor cores (FP32 build)
    Method method = METHOD_DIRECT;
    // DIRECT
    std::vector<PassSpec> passes;
    const vec2_t* tw_lo = nullptr;
    const vec2_t* tw_hi = nullptr;
    uint32_t tw_shift = 0;
    // RADER / BLUESTEIN: the convolution length and its two DIRECT sub-plans
    uint32_t L = 0;
    FftPlan* sub_fwd = nullptr;
    FftPlan* sub_inv = nullptr;
    const vec2_t* chirp = nullptr;   // Bluestein
    const vec2_t* spectrum = nullptr; // Bluestein filter / Rader kernel spectrum, 1/L folded in
    const uint32_t* gperm = nullptr;  // Rader: g^j mod p
    const uint32_t* iperm = nullptr;  // Rader: g^-j mod p
    uint32_t generator = 0;
    ~FftPlan();
};

// Element layout of a batch of sequences.
struct Layout {
    uint32_t batch = 1;
    uint64_t bs = 0;  // batch stride (elements)
    uint32_t es = 1;  // element stride
    uint8_t order = ORDER_J;
};

// Bump allocator over a caller-provided device workspace.
struct Workspace {
    char* base = nullptr;
    size_t size = 0;
    size_t used = 0;
    vec2_t* take(size_t elems);
};

struct DeviceArena {
    std::vector<void*> blocks;
    size_t bytes = 0;
    void* alloc(size_t bytes);
    ~DeviceArena();
};

// Builds the plan of an N-point transform of direction `sign` on the current
// device, allocating its tables from `arena`.  Returns nullptr on failure.
FftPlan* make_plan(uint32_t N, int sign, DeviceArena& arena, cudaStream_t st,
                   uint32_t max_prime = kMaxDirectPrime, const PlanVariant& var = PlanVariant());
bool is_direct_length(uint32_t n, uint32_t max_prime = kMaxDirectPrime);
// Marks a plan tree to run its radix-16 passes on tensor cores (FP32 build).
void set_tensor_cores(FftPlan* p, bool on);
std::string describe(const FftPlan& p);
// Device workspace (bytes) the plan needs for `batch` sequences.
size_t workspace_bytes(const FftPlan& p, uint32_t batch);
// Appends the passes computing out = FFT(in) * scale to `descs`.
bool build_passes(const FftPlan& p, const vec2_t* in, const Layout& lin, vec2_t* out,
                  const Layout& lout, real_t scale, Workspace& ws, std::vector<PassDesc>& descs);
void run_passes(const std::vector<PassDesc>& descs, cudaStream_t st);
// Descriptor of pass `pass` of a DIRECT plan (no fused element operations).
// Start of chunk i (i = 0..k; chunk k's start is `total`) when `total` units
// are split into k chunks for a host-buffer pipeline: the first and last
// chunks get a quarter of the share of the others, because the copy in of
// the first and the transform and copy out of the last overlap nothing.
// Starts strictly increase when total >= 2k.
inline uint64_t chunk_start(uint64_t i, uint64_t k, uint64_t total) {
    if (i == 0) return 0;
    if (i >= k) return total;
    if (k < 3 || total < 2 * k) return total * i / k;
    // weights 1/4, 1, ..., 1, 1/4 in quarters: 1, 4, ..., 4, 1
    const uint64_t quarters = 4 * (k - 2) + 2;
    const uint64_t before = 1 + 4 * (i - 1);
    uint64_t s = total * before / quarters;
    return s < i ? i : s;
}

// Copy ranges of a chunked host-buffer call on 256-byte boundaries: copies
// that start or end off a 128-byte boundary cut the host link's two-way
// throughput from about 338 to 250 GB/s on this hardware.  The copy in of a
// chunk rounds its start up and the copy out rounds it down, so the transform
// of every chunk finds its input copied (by its own copy in or the one
// before, on the same stream) and every copy out reads finished output only.
// [b0, b1) is the chunk's byte range; first/last chunks reach 0 and `total`.
struct CopyRange {
    size_t in0, in1, out0, out1;
};
inline CopyRange copy_range(size_t b0, size_t b1, size_t total, bool first, bool last) {
    auto up = [&](size_t b) { return std::min(total, (b + 255) & ~size_t(255)); };
    auto down = [](size_t b) { return b & ~size_t(255); };
    CopyRange r;
    r.in0 = first ? 0 : up(b0);
    r.in1 = last ? total : up(b1);
    r.out0 = first ? 0 : down(b0);
    r.out1 = last ? total : down(b1);
    return r;
}

// Shared-memory slots from one lane to the next in a compile-time
// (power-of-two) tile body of C lanes of R points run by `threads` threads:
// the padded lane plus the skew with the fewest bank conflicts.
uint32_t spec_lane_stride(uint32_t R, uint32_t C, bool load_lane, bool store_lane,
                          uint32_t threads);
// true when every pass of a direct plan run down the columns of a row-major
// array gets tiles of four columns or more (32-byte row segments)
bool columns_coalesce(const FftPlan& P);
PassDesc make_pass_desc(const FftPlan& P, size_t pass, const vec2_t* in, const Layout& lin,
                        vec2_t* out, const Layout& lout, real_t scale);

// The device plan behind a public complex plan handle (nullptr if none).
const FftPlan* device_plan_of(const kfft_plan_cpx* p);

// ---- runtime ----------------------------------------------------------------
// Bounded device waits that can run out (the bulk-copy waits of k_pass_bulk)
// record the failure in a per-host-thread slot of a device array.
constexpr int kWaitSlots = 64;
// Polls of a bulk-copy wait before it gives up (about a second of try_wait
// suspensions); a test hook can lower it.
constexpr uint32_t kBulkMaxPolls = 1u << 22;
int wait_slot();
// After the work queued on `st` is done: reads and clears this thread's slot;
// true when a wait ran out since the last check.
bool take_wait_failures(cudaStream_t st);
// Records an engine failure that is not a CUDA error (for kfft_gb300_last_error).
void note_engine_error(const char* msg);
int current_device();
bool ensure_device();
void note_cuda_error(cudaError_t e);
// returns and clears the CUDA error recorded on this host thread since the last call
int take_pending_error();
void count_launch(int64_t n = 1);
void count_graph_launch();
void account_device_bytes(int64_t delta);

}  // namespace kfft
