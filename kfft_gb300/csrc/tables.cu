// tables.cu -- FP64 table generation (twiddles, chirps, Rader kernels, real
// post-twiddles) and the small elementwise/layout kernels of the engine.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.cuh"

namespace kfft {

__device__ __forceinline__ vec2_t cmul_t(vec2_t a, vec2_t b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ vec2_t cadd_t(vec2_t a, vec2_t b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ vec2_t csub_t(vec2_t a, vec2_t b) { return {a.x - b.x, a.y - b.y}; }

void FastDiv::init(uint32_t div) {
    d = div ? div : 1;
    uint32_t l = 0;
    while (l < 32 && (uint64_t(1) << l) < d) ++l;
    s = l;
    // m = floor(2^32 * (2^l - d) / d) + 1  (fits in 32 bits for d >= 1)
    m = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d + 1);
}

// ---------------------------------------------------------------------------
// FP64 table generation
// ---------------------------------------------------------------------------
__global__ void k_gen_twiddles(vec2_t* t, uint32_t count, uint64_t mult, uint32_t n, int sign) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += gridDim.x * blockDim.x) {
        uint64_t e = (uint64_t(i) * mult) % n;
        int64_t es = (2 * e > n) ? int64_t(e) - int64_t(n) : int64_t(e);
        double s, c;
        sincospi(2.0 * double(es) / double(n), &s, &c);
        t[i] = {real_t(c), real_t(sign * s)};
    }
}

void gen_twiddles(vec2_t* t, uint32_t count, uint64_t mult, uint32_t n, int sign,
                  cudaStream_t st) {
    if (!count) return;
    uint32_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_gen_twiddles<<<blocks, 256, 0, st>>>(t, count, mult, n, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_gen_chirp(vec2_t* c, uint32_t count, uint32_t n, int sign) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count;
         k += gridDim.x * blockDim.x) {
        const uint64_t two_n = 2 * uint64_t(n);
        uint64_t kk = k % two_n;
        uint64_t e = (kk * kk) % two_n;  // k^2 mod 2n, exact in integers
        int64_t es = (e > n) ? int64_t(e) - int64_t(two_n) : int64_t(e);
        double s, co;
        sincospi(double(es) / double(n), &s, &co);
        c[k] = {real_t(co), real_t(sign * s)};
    }
}

void gen_chirp(vec2_t* c, uint32_t count, uint32_t n, int sign, cudaStream_t st) {
    uint32_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_gen_chirp<<<blocks, 256, 0, st>>>(c, count, n, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_bluestein_filter(vec2_t* b, const vec2_t* chirp, uint32_t n, uint32_t m_len) {
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < m_len;
         m += gridDim.x * blockDim.x) {
        vec2_t v = {real_t(0), real_t(0)};
        if (m < n) v = chirp[m];
        else if (m > m_len - n) v = chirp[m_len - m];
        b[m] = {v.x, -v.y};
    }
}

void gen_bluestein_filter(vec2_t* b, const vec2_t* chirp, uint32_t n, uint32_t m_len,
                          cudaStream_t st) {
    uint32_t blocks = (m_len + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_bluestein_filter<<<blocks, 256, 0, st>>>(b, chirp, n, m_len);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_gen_rader(vec2_t* s, const uint32_t* pidx, uint32_t p, int sign) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j + 1 < p;
         j += gridDim.x * blockDim.x) {
        uint32_t e = pidx[j];
        int64_t es = (2 * uint64_t(e) > p) ? int64_t(e) - int64_t(p) : int64_t(e);
        double sn, c;
        sincospi(2.0 * double(es) / double(p), &sn, &c);
        s[j] = {real_t(c), real_t(sign * sn)};
    }
}

void gen_rader_kernel(vec2_t* s, const uint32_t* pidx, uint32_t p, int sign, cudaStream_t st) {
    uint32_t blocks = (p + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_gen_rader<<<blocks, 256, 0, st>>>(s, pidx, p, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_super_twiddles(vec2_t* t, uint32_t h, int sign) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < h; k += gridDim.x * blockDim.x) {
        // phase = sign * pi * ((k+1)/h + 1/2) = sign * pi * (2(k+1) + h) / (2h)
        uint64_t num = (2 * uint64_t(k + 1) + h) % (4 * uint64_t(h));
        int64_t ns = (num > 2 * uint64_t(h)) ? int64_t(num) - int64_t(4 * uint64_t(h)) : int64_t(num);
        double s, c;
        sincospi(double(ns) / (2.0 * double(h)), &s, &c);
        t[k] = {real_t(c), real_t(sign * s)};
    }
}

void gen_super_twiddles(vec2_t* t, uint32_t h, int sign, cudaStream_t st) {
    if (!h) return;
    uint32_t blocks = (h + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_super_twiddles<<<blocks, 256, 0, st>>>(t, h, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_scale_table(vec2_t* t, uint32_t count, double s) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += gridDim.x * blockDim.x)
        t[i] = {real_t(t[i].x * s), real_t(t[i].y * s)};
}

void scale_table(vec2_t* t, uint32_t count, double s, cudaStream_t st) {
    uint32_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_scale_table<<<blocks, 256, 0, st>>>(t, count, s);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// ---------------------------------------------------------------------------
// real transform post/pre processing (kfft_scalar.c:174-242)
// ---------------------------------------------------------------------------
// The bins of the even-N real forward transform from the N/2-point spectrum
// z (kfft_scalar.c:174-216); with `mul`, each stored bin is multiplied by the
// same bin of mul (a convolution's other spectrum, same layout as out).
__global__ void k_real_post(const vec2_t* __restrict__ z, vec2_t* __restrict__ out,
                            const vec2_t* __restrict__ stt, uint32_t h, uint32_t batch,
                            uint64_t out_bs, int expand, const vec2_t* __restrict__ mul) {
    const uint32_t half = h / 2;  // k = 1..half
    const uint64_t per = uint64_t(half) + 1;
    const uint64_t total = per * batch;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t b = uint32_t(t / per);
        const uint32_t k = uint32_t(t - uint64_t(b) * per);
        const vec2_t* Z = z + uint64_t(b) * h;
        vec2_t* O = out + uint64_t(b) * out_bs;
        const vec2_t* M = mul ? mul + uint64_t(b) * out_bs : nullptr;
        // store bin i (times mul's bin i when fused with a convolution product)
        auto put = [&](uint32_t i, vec2_t v) { O[i] = M ? cmul_t(v, M[i]) : v; };
        const uint32_t n = 2 * h;
        if (k == 0) {
            vec2_t z0 = Z[0];
            put(0, {z0.x + z0.y, real_t(0)});
            put(h, {z0.x - z0.y, real_t(0)});
            continue;
        }
        vec2_t fpk = Z[k];
        vec2_t zn = Z[h - k];
        vec2_t fpnk = {zn.x, -zn.y};
        vec2_t f1k = cadd_t(fpk, fpnk), f2k = csub_t(fpk, fpnk);
        vec2_t tw = cmul_t(f2k, stt[k - 1]);
        vec2_t a = {real_t(0.5) * (f1k.x + tw.x), real_t(0.5) * (f1k.y + tw.y)};
        vec2_t bb = {real_t(0.5) * (f1k.x - tw.x), real_t(0.5) * (tw.y - f1k.y)};
        if (2 * k == h) {
            put(k, bb);  // both values land on the same bin; the later one wins
            if (expand) put(n - k, {bb.x, -bb.y});
        } else {
            put(k, a);
            put(h - k, bb);
            if (expand) {
                put(n - k, {a.x, -a.y});
                put(n - (h - k), {bb.x, -bb.y});
            }
        }
    }
}

void launch_real_post(const vec2_t* z, vec2_t* out, const vec2_t* st_tab, uint32_t h,
                      uint32_t batch, uint64_t out_bs, int expand, cudaStream_t st,
                      const vec2_t* mul) {
    uint64_t total = (uint64_t(h / 2) + 1) * batch;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_real_post<<<uint32_t(blocks), 256, 0, st>>>(z, out, st_tab, h, batch, out_bs, expand, mul);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_real_pre(const vec2_t* __restrict__ in, vec2_t* __restrict__ z,
                           const vec2_t* __restrict__ stt, uint32_t h, uint32_t batch,
                           uint64_t in_bs) {
    const uint32_t half = h / 2;
    const uint64_t per = uint64_t(half) + 1;
    const uint64_t total = per * batch;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t b = uint32_t(t / per);
        const uint32_t k = uint32_t(t - uint64_t(b) * per);
        const vec2_t* I = in + uint64_t(b) * in_bs;
        vec2_t* Z = z + uint64_t(b) * h;
        if (k == 0) {
            Z[0] = {I[0].x + I[h].x, I[0].x - I[h].x};
            continue;
        }
        vec2_t fk = I[k];
        vec2_t fn = I[h - k];
        vec2_t fnkc = {fn.x, -fn.y};
        vec2_t fek = cadd_t(fk, fnkc), tmp = csub_t(fk, fnkc);
        vec2_t fok = cmul_t(tmp, stt[k - 1]);
        vec2_t lo = cadd_t(fek, fok);
        vec2_t hi = csub_t(fek, fok);
        hi.y = -hi.y;
        if (2 * k == h) {
            Z[k] = hi;
        } else {
            Z[k] = lo;
            Z[h - k] = hi;
        }
    }
}

void launch_real_pre(const vec2_t* in, vec2_t* z, const vec2_t* st_tab, uint32_t h,
                     uint32_t batch, uint64_t in_bs, cudaStream_t st) {
    uint64_t total = (uint64_t(h / 2) + 1) * batch;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_real_pre<<<uint32_t(blocks), 256, 0, st>>>(in, z, st_tab, h, batch, in_bs);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// The same pre-processing down the columns of a row-major array: sequence c
// is column c (element k at row k), of `ncols` columns; row strides in_rs and
// z_rs.  Consecutive threads take consecutive columns.
__global__ void k_real_pre_cols(const vec2_t* __restrict__ in, vec2_t* __restrict__ z,
                                const vec2_t* __restrict__ stt, uint32_t h, uint32_t ncols,
                                uint64_t in_rs, uint64_t z_rs) {
    const uint32_t half = h / 2;
    const uint64_t total = (uint64_t(half) + 1) * ncols;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t k = uint32_t(t / ncols);
        const uint32_t c = uint32_t(t - uint64_t(k) * ncols);
        auto I = [&](uint32_t r) { return in[uint64_t(r) * in_rs + c]; };
        vec2_t* Z = z + c;
        if (k == 0) {
            const vec2_t a = I(0), b = I(h);
            Z[0] = {a.x + b.x, a.x - b.x};
            continue;
        }
        vec2_t fk = I(k);
        vec2_t fn = I(h - k);
        vec2_t fnkc = {fn.x, -fn.y};
        vec2_t fek = cadd_t(fk, fnkc), tmp = csub_t(fk, fnkc);
        vec2_t fok = cmul_t(tmp, stt[k - 1]);
        vec2_t lo = cadd_t(fek, fok);
        vec2_t hi = csub_t(fek, fok);
        hi.y = -hi.y;
        if (2 * k == h) {
            Z[uint64_t(k) * z_rs] = hi;
        } else {
            Z[uint64_t(k) * z_rs] = lo;
            Z[uint64_t(h - k) * z_rs] = hi;
        }
    }
}

void launch_real_pre_cols(const vec2_t* in, vec2_t* z, const vec2_t* st_tab, uint32_t h,
                          uint32_t ncols, uint64_t in_rs, uint64_t z_rs, cudaStream_t st) {
    uint64_t total = (uint64_t(h / 2) + 1) * ncols;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_real_pre_cols<<<uint32_t(blocks), 256, 0, st>>>(in, z, st_tab, h, ncols, in_rs, z_rs);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// Column-wise complex results of h rows to 2h real rows: row 2m gets the real
// parts of row m, row 2m+1 its imaginary parts (the even-length real inverse
// run down the columns).
__global__ void k_split_rows(const vec2_t* __restrict__ z, real_t* __restrict__ out, uint32_t h,
                             uint32_t ncols) {
    const uint64_t total = uint64_t(h) * ncols;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t m = t / ncols, c = t - m * ncols;
        const vec2_t v = z[t];
        out[(2 * m) * ncols + c] = v.x;
        out[(2 * m + 1) * ncols + c] = v.y;
    }
}

void launch_split_rows(const vec2_t* z, real_t* out, uint32_t h, uint32_t ncols, cudaStream_t st) {
    uint64_t total = uint64_t(h) * ncols;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_split_rows<<<uint32_t(blocks), 256, 0, st>>>(z, out, h, ncols);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// Bins x/2+1 .. x-1 of each row of a y-by-x 2D spectrum of real data from
// the computed half: X[k1][k2] = conj(X[(y - k1) mod y][x - k2]) (x even).
__global__ void k_hermitian_fill(vec2_t* __restrict__ data, uint32_t x, uint32_t y) {
    const uint32_t w = x / 2 - 1;  // filled bins per row
    const uint64_t total = uint64_t(w) * y;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t k1 = uint32_t(t / w);
        const uint32_t k2 = x / 2 + 1 + uint32_t(t - uint64_t(k1) * w);
        const uint32_t r = k1 ? y - k1 : 0;
        const vec2_t v = data[uint64_t(r) * x + (x - k2)];
        data[uint64_t(k1) * x + k2] = {v.x, -v.y};
    }
}

void launch_hermitian_fill(vec2_t* data, uint32_t x, uint32_t y, cudaStream_t st) {
    const uint64_t total = uint64_t(x / 2 - 1) * y;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_hermitian_fill<<<uint32_t(blocks), 256, 0, st>>>(data, x, y);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_widen(const real_t* __restrict__ in, vec2_t* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        out[i] = {in[i], real_t(0)};
}
void launch_widen(const real_t* in, vec2_t* out, uint64_t n, cudaStream_t st) {
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_widen<<<uint32_t(blocks), 256, 0, st>>>(in, out, n);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_narrow(const vec2_t* __restrict__ in, real_t* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        out[i] = in[i].x;
}
void launch_narrow(const vec2_t* in, real_t* out, uint64_t n, cudaStream_t st) {
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_narrow<<<uint32_t(blocks), 256, 0, st>>>(in, out, n);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// 32x32 tiled transpose: out[b][c][r] = in[b][r][c]
template <typename E>
__global__ void k_transpose(const E* __restrict__ in, E* __restrict__ out, uint32_t rows,
                            uint32_t cols) {
    __shared__ E tile[32][33];
    const uint64_t boff = uint64_t(blockIdx.z) * rows * cols;
    const uint32_t c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
        uint32_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[i][threadIdx.x] = in[boff + uint64_t(r) * cols + c];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
        uint32_t c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[boff + uint64_t(c) * rows + r] = tile[threadIdx.x][i];
    }
}

void launch_transpose(const vec2_t* in, vec2_t* out, uint32_t rows, uint32_t cols,
                      uint32_t batch, cudaStream_t st) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32, batch);
    k_transpose<vec2_t><<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

void launch_transpose_real(const real_t* in, real_t* out, uint32_t rows, uint32_t cols,
                           cudaStream_t st) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32, 1);
    k_transpose<real_t><<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_hadamard(vec2_t* __restrict__ b, const vec2_t* __restrict__ a, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        b[i] = cmul_t(b[i], a[i]);
}

void launch_hadamard(vec2_t* b, const vec2_t* a, uint64_t n, cudaStream_t st) {
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_hadamard<<<uint32_t(blocks), 256, 0, st>>>(b, a, n);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_copy_rows(const vec2_t* __restrict__ in, vec2_t* __restrict__ out, uint32_t len,
                            uint64_t ss, uint64_t ds, uint32_t rows) {
    const uint64_t total = uint64_t(len) * rows;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        uint64_t r = t / len, c = t - r * len;
        out[r * ds + c] = in[r * ss + c];
    }
}

void launch_copy_rows(const vec2_t* in, vec2_t* out, uint32_t len, uint64_t src_stride,
                      uint64_t dst_stride, uint32_t rows, cudaStream_t st) {
    uint64_t total = uint64_t(len) * rows;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_copy_rows<<<uint32_t(blocks), 256, 0, st>>>(in, out, len, src_stride, dst_stride, rows);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

}  // namespace kfft
