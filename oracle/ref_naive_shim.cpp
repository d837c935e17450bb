// C entry point around the reference's own scalar CSR SpMM (cpp_testbed/src/spmm/baselines/
// spmm_naive.cpp:3-28), which this recipe compiles unchanged from the reference checkout.
// Test infrastructure: used only to pin the oracle against the reference's FP32 arithmetic.
#include "spmm.h"

void spmm_naive(int m, int k, int n, int nonzeros, const int *row_indices, const float *values,
                const int *row_offsets, const int *column_indices, const float *dense_matrix, float *output_matrix,
                int batch_size, const NullConfig &config);

extern "C" void ref_spmm_naive(int m, int k, int n, int nnz, const float *values, const int *row_offsets,
                               const int *col_inds, const float *B, float *C) {
    NullConfig cfg;
    spmm_naive(m, k, n, nnz, nullptr, values, row_offsets, col_inds, B, C, 1, cfg);
}
