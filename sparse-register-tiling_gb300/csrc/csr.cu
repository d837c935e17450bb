// csr.cu -- the reference's CSR baseline SpMM on the GPU: csr.executor of
// sbench/SOP/_C/pytorch_csr_wrapper.cpp:314-353 (kernel :70-191), which sbench/SOP/sop_bench.py:197
// times beside the register-tiled executor.
//
// One warp per (row, strip of 32 * NV columns); lane l keeps NV consecutive columns of the row in
// registers.  The row's nonzeros are read 32 at a time, one (column, value) per lane with coalesced
// loads, and handed to the whole warp by shuffles; each nonzero then costs one NV-float load of its
// B row per lane.  FMAs run in CSR order from zero, so every C element is the same fmaf chain as the
// reference's row x N-tile loop, whatever the tile: results are bit-identical to the oracle's.
#include "spreg_common.cuh"

#include <algorithm>
#include <vector>

namespace spreg {

// Reads stay in bounds whatever the CSR holds: row pointers are clamped to [0, nnz] and a column
// index outside [0, k) contributes nothing and sets the device status word (code 20).
constexpr int kCsrBadIndex = 20;

template <int NV>
__global__ void __launch_bounds__(256) csr_spmm_kernel(const int64_t M, const int64_t k_rows, const int64_t n,
                                                       const int64_t nnz, const int32_t *__restrict__ row_ptrs,
                                                       const int32_t *__restrict__ col_inds,
                                                       const float *__restrict__ values, const float *__restrict__ B,
                                                       const int64_t ldb, float *__restrict__ C, const int64_t ldc,
                                                       const bool vec, int *status) {
    const int lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= M) return;
    const int64_t col0 = (int64_t)blockIdx.y * (32 * NV) + (int64_t)lane * NV;
    const bool whole = vec && col0 + NV <= n;  // this lane's NV columns exist and load as one vector
    float acc[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = 0.0f;
    int64_t p0 = row_ptrs[row], p1 = row_ptrs[row + 1];
    p0 = p0 < 0 ? 0 : (p0 > nnz ? nnz : p0);
    p1 = p1 < p0 ? p0 : (p1 > nnz ? nnz : p1);
    for (int64_t base = p0; base < p1; base += 32) {
        const int64_t p = base + lane;
        int32_t my_k = p < p1 ? __ldg(col_inds + p) : 0;
        float my_a = p < p1 ? __ldg(values + p) : 0.0f;
        if (my_k < 0 || my_k >= k_rows) {
            if (p < p1 && status) atomicCAS(status, 0, kCsrBadIndex);
            my_k = -1;
        }
        const int cnt = (p1 - base) < 32 ? (int)(p1 - base) : 32;
        for (int q = 0; q < cnt; ++q) {
            const int32_t k = __shfl_sync(0xffffffffu, my_k, q);
            const float a = __shfl_sync(0xffffffffu, my_a, q);
            if (k < 0) continue;  // warp-uniform: every lane holds the same k
            const float *b = B + (int64_t)k * ldb + col0;
            float bv[NV];
            if (whole) {
                if constexpr (NV == 1) {
                    bv[0] = __ldg(b);
                } else if constexpr (NV == 2) {
                    const float2 t = __ldg(reinterpret_cast<const float2 *>(b));
                    bv[0] = t.x; bv[1] = t.y;
                } else {
                    const float4 t = __ldg(reinterpret_cast<const float4 *>(b));
                    bv[0] = t.x; bv[1] = t.y; bv[2] = t.z; bv[3] = t.w;
                }
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) bv[j] = col0 + j < n ? __ldg(b + j) : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < NV; ++j) acc[j] = fmaf(a, bv[j], acc[j]);
        }
    }
    float *c = C + row * ldc + col0;
#pragma unroll
    for (int j = 0; j < NV; ++j)
        if (col0 + j < n) c[j] = acc[j];
}

int *device_status_word(int *st);  // exec.cu

namespace {

// n_tile (the reference's register tile, 16 / 32 / 64 / 128 floats) -> columns per lane.
int csr_nv(int32_t n_tile) { return n_tile <= 32 ? 1 : (n_tile == 64 ? 2 : 4); }

int csr_launch(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs, const int32_t *col_inds,
               const float *values, const float *b, int64_t ldb, float *c, int64_t ldc, int nv, cudaStream_t stream) {
    if (rows == 0 || n == 0) return SPREG_OK;
    int st = SPREG_OK;
    int *status = device_status_word(&st);
    if (st) return st;
    const bool vec = ((uintptr_t)b % (4 * nv)) == 0 && ldb % nv == 0;
    const int64_t strips = (n + 32 * nv - 1) / (32 * nv);
    SPREG_CHECK_ARG(strips <= 65535, "n too large for one launch");
    const dim3 grid((unsigned)((rows + 7) / 8), (unsigned)strips);
    switch (nv) {
    case 1:
        csr_spmm_kernel<1><<<grid, 256, 0, stream>>>(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc,
                                                     vec, status);
        break;
    case 2:
        csr_spmm_kernel<2><<<grid, 256, 0, stream>>>(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc,
                                                     vec, status);
        break;
    default:
        csr_spmm_kernel<4><<<grid, 256, 0, stream>>>(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc,
                                                     vec, status);
        break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "csr launch: %s", cudaGetErrorString(e));
    return SPREG_OK;
}

int csr_check(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs, const int32_t *col_inds,
              const float *values, const float *b, int64_t ldb, const float *c, int64_t ldc, int32_t n_tile) {
    SPREG_CHECK_ARG(rows >= 0 && cols >= 0 && n >= 0 && nnz >= 0, "negative size");
    SPREG_CHECK_ARG(rows <= INT32_MAX - 1 && cols <= INT32_MAX && nnz <= INT32_MAX, "size out of range");
    SPREG_CHECK_ARG(n_tile == 16 || n_tile == 32 || n_tile == 64 || n_tile == 128,
                    "n_tile must be 16, 32, 64 or 128 (pytorch_csr_wrapper.cpp:258-271), got %d", n_tile);
    SPREG_CHECK_ARG(ldb >= n && ldc >= n, "ldb / ldc below n");
    SPREG_CHECK_ARG(rows == 0 || n == 0 || (row_ptrs && c), "null row_ptrs or C");
    SPREG_CHECK_ARG(rows == 0 || n == 0 || nnz == 0 || (col_inds && values && b), "null CSR arrays or B");
    return SPREG_OK;
}

}  // namespace

int csr_spmm_impl(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs,
                  const int32_t *col_inds, const float *values, const float *b, int64_t ldb, float *c, int64_t ldc,
                  int32_t n_tile, cudaStream_t stream) {
    int st = csr_check(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, n_tile);
    if (st) return st;
    return csr_launch(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, csr_nv(n_tile), stream);
}

// profile() of pytorch_csr_wrapper.cpp:200-232: num_runs warm-up runs, then 150 iterations of
// num_runs runs; the median per run (CUDA events on `stream`).
int csr_spmm_timed_impl(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs,
                        const int32_t *col_inds, const float *values, const float *b, int64_t ldb, float *c,
                        int64_t ldc, int32_t n_tile, int64_t num_runs, double *median_ns, cudaStream_t stream) {
    int st = csr_check(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, n_tile);
    if (st) return st;
    SPREG_CHECK_ARG(median_ns && num_runs >= 1, "null median_ns or num_runs < 1");
    const int nv = csr_nv(n_tile);
    for (int64_t r = 0; r < num_runs; ++r)
        if ((st = csr_launch(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, nv, stream))) return st;
    const int kIters = 150;
    std::vector<cudaEvent_t> ev(2 * kIters);
    for (auto &e : ev) SPREG_CUDA(cudaEventCreate(&e));
    for (int it = 0; it < kIters && !st; ++it) {
        cudaEventRecord(ev[2 * it], stream);
        for (int64_t r = 0; r < num_runs && !st; ++r)
            st = csr_launch(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, nv, stream);
        cudaEventRecord(ev[2 * it + 1], stream);
    }
    cudaError_t e = cudaStreamSynchronize(stream);
    std::vector<double> t(kIters);
    for (int it = 0; it < kIters && e == cudaSuccess; ++it) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[2 * it], ev[2 * it + 1]);
        t[it] = ms * 1e6 / (double)num_runs;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (st) return st;
    if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "timed csr: %s", cudaGetErrorString(e));
    std::sort(t.begin(), t.end());
    *median_ns = (t[kIters / 2 - 1] + t[kIters / 2]) / 2.0;
    return SPREG_OK;
}

}  // namespace spreg
