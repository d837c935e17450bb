/*
 * spreg_cpu_fast.c -- the reference's register-tiled executor as SIMD code for the host CPU: the
 * timed CPU baseline of the benchmark.
 *
 * TEST INFRASTRUCTURE ONLY.  Only bench.py's CPU baseline / reference arm and tests/ load it (as
 * part of liboracle.so); the product (libspreg.so) never calls it.
 *
 * It runs the same packed arena as the checker's executor (orc_execute in spreg_oracle.c) with the
 * structure of the reference's generated microkernels (tools/codegen/gen_vector_specialized.py:
 * 266-357, executor loop sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305): per row panel
 * and strip of N_r columns, M_r x N_r accumulators held in vector registers, and for every
 * nanokernel id a loop over its count entries that loads one B row segment and issues the pattern's
 * FMAs -- the rows of the pattern fixed at compile time, one case per pattern, as the reference's
 * code generator emits one routine per nanokernel.  N_r = 16 floats (four 128-bit vectors per row);
 * OpenMP threads split the row panels.
 *
 * Every output element is the same FMA chain in packed-entry order as the checker: vector
 * expressions acc + a * b are contracted to fused multiply-adds (-ffp-contract=fast), lane by lane
 * the fmaf() of the checker, so results are bit-identical to it.  Only FP32 values, B and C, M_r
 * <= 8; the CPU baseline workloads are FP32.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t values_off, cols_off, counts_off;
    int32_t num_values, num_cols;
} fast_desc; /* same layout as spreg_panel_desc */

typedef float v16 __attribute__((vector_size(64)));

/* Descriptor index of (global panel gp, K tile tj): units are ordered row tile, K tile, panel. */
static int64_t fast_unit(int64_t gp, int64_t tj, int64_t ppt, int64_t T, int64_t P) {
    int64_t ti = gp / ppt, p = gp % ppt;
    int64_t p_lo = ti * ppt;
    int64_t n_in = (p_lo + ppt < P ? ppt : P - p_lo);
    return p_lo * T + tj * n_in + p;
}

static inline v16 ld16(const float *p) {
    v16 v;
    memcpy(&v, p, sizeof v);
    return v;
}
static inline void st16(float *p, v16 v) { memcpy(p, &v, sizeof v); }
static inline v16 relu16(v16 v) { /* fmaxf(o, 0), as the checker's epilogue */
    float t[16];
    memcpy(t, &v, sizeof t);
    for (int j = 0; j < 16; ++j) t[j] = fmaxf(t[j], 0.0f);
    memcpy(&v, t, sizeof t);
    return v;
}

/* One nanokernel group of an M_r <= 4 panel: n entries of pattern P (compile-time constant). */
#define GROUP4(P)                                                                                  \
    case P:                                                                                        \
        for (int32_t e = 0; e < n; ++e) {                                                          \
            const v16 b = ld16(B + (int64_t)cols[c++] * ldb + j0);                                 \
            if ((P) & 1) a0 += vp[v++] * b;                                                        \
            if ((P) & 2) a1 += vp[v++] * b;                                                        \
            if ((P) & 4) a2 += vp[v++] * b;                                                        \
            if ((P) & 8) a3 += vp[v++] * b;                                                        \
        }                                                                                          \
        break;

static void panel_mr4(int num_nkern, const int32_t *id_to_pattern, const uint8_t *arena, const fast_desc *descs,
                      int64_t gp, int64_t M, int64_t P, int64_t ppt, int64_t T, const float *B, int64_t ldb, float *C,
                      int64_t ldc, int64_t N, int load_c, int epilogue, int mr) {
    for (int64_t j0 = 0; j0 + 16 <= N; j0 += 16) {
        v16 a0 = {0}, a1 = {0}, a2 = {0}, a3 = {0};
        const int64_t r0 = gp * mr;
        if (load_c) {
            if (r0 + 0 < M) a0 = ld16(C + (r0 + 0) * ldc + j0);
            if (mr > 1 && r0 + 1 < M) a1 = ld16(C + (r0 + 1) * ldc + j0);
            if (mr > 2 && r0 + 2 < M) a2 = ld16(C + (r0 + 2) * ldc + j0);
            if (mr > 3 && r0 + 3 < M) a3 = ld16(C + (r0 + 3) * ldc + j0);
        }
        for (int64_t tj = 0; tj < T; ++tj) {
            const fast_desc *d = &descs[fast_unit(gp, tj, ppt, T, P)];
            const int32_t *cnt = (const int32_t *)(arena + d->counts_off);
            const int32_t *cols = (const int32_t *)(arena + d->cols_off);
            const float *vp = (const float *)(arena + d->values_off);
            int64_t c = 0, v = 0;
            for (int id = 0; id < num_nkern; ++id) {
                const int32_t n = cnt[id];
                if (n == 0) continue;
                switch (id_to_pattern[id]) {
                    GROUP4(1) GROUP4(2) GROUP4(3) GROUP4(4) GROUP4(5) GROUP4(6) GROUP4(7) GROUP4(8)
                    GROUP4(9) GROUP4(10) GROUP4(11) GROUP4(12) GROUP4(13) GROUP4(14) GROUP4(15)
                default: break;
                }
            }
        }
        v16 out[4] = {a0, a1, a2, a3};
        for (int r = 0; r < mr; ++r) {
            if (r0 + r >= M) continue;
            v16 o = out[r];
            if (epilogue == 1) o = relu16(o);
            st16(C + (r0 + r) * ldc + j0, o);
        }
    }
}

/* Any M_r <= 8: the rows of each group's pattern in a small list (runtime); used for M_r > 4. */
static void panel_generic(int mr, int num_nkern, const int32_t *id_to_pattern, const uint8_t *arena,
                          const fast_desc *descs, int64_t gp, int64_t M, int64_t P, int64_t ppt, int64_t T,
                          const float *B, int64_t ldb, float *C, int64_t ldc, int64_t N, int load_c, int epilogue) {
    for (int64_t j0 = 0; j0 + 16 <= N; j0 += 16) {
        v16 acc[8];
        const int64_t r0 = gp * mr;
        for (int r = 0; r < mr; ++r) {
            const v16 z = {0};
            acc[r] = (load_c && r0 + r < M) ? ld16(C + (r0 + r) * ldc + j0) : z;
        }
        for (int64_t tj = 0; tj < T; ++tj) {
            const fast_desc *d = &descs[fast_unit(gp, tj, ppt, T, P)];
            const int32_t *cnt = (const int32_t *)(arena + d->counts_off);
            const int32_t *cols = (const int32_t *)(arena + d->cols_off);
            const float *vp = (const float *)(arena + d->values_off);
            int64_t c = 0, v = 0;
            for (int id = 0; id < num_nkern; ++id) {
                const int32_t n = cnt[id];
                const uint32_t pat = (uint32_t)id_to_pattern[id];
                int rows[8], nr = 0;
                for (int r = 0; r < mr; ++r)
                    if ((pat >> r) & 1u) rows[nr++] = r;
                for (int32_t e = 0; e < n; ++e) {
                    const v16 b = ld16(B + (int64_t)cols[c++] * ldb + j0);
                    for (int q = 0; q < nr; ++q) acc[rows[q]] += vp[v++] * b;
                }
            }
        }
        for (int r = 0; r < mr; ++r) {
            if (r0 + r >= M) continue;
            v16 o = acc[r];
            if (epilogue == 1) o = relu16(o);
            st16(C + (r0 + r) * ldc + j0, o);
        }
    }
}

/* C (+)= A . B for FP32 values, B and C, over the first N columns; N must be a multiple of 16
 * (returns -1 otherwise, and for M_r > 8).  Same arguments as orc_execute. */
int orc_execute_fast(int mr, int num_nkern, const int32_t *id_to_pattern, const uint8_t *arena,
                     const fast_desc *descs, int64_t M, int64_t P, int64_t ppt, int64_t T, const float *B, int64_t ldb,
                     float *C, int64_t ldc, int64_t N, int load_c, int epilogue, int num_threads) {
    if (mr < 1 || mr > 8 || N % 16 != 0) return -1;
#ifdef _OPENMP
    if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(num_threads)
#endif
    for (int64_t gp = 0; gp < P; ++gp) {
        if (mr <= 4)
            panel_mr4(num_nkern, id_to_pattern, arena, descs, gp, M, P, ppt, T, B, ldb, C, ldc, N, load_c, epilogue,
                      mr);
        else
            panel_generic(mr, num_nkern, id_to_pattern, arena, descs, gp, M, P, ppt, T, B, ldb, C, ldc, N, load_c,
                          epilogue);
    }
    return 0;
}

/* The reference's CSR baseline (sbench/SOP/_C/pytorch_csr_wrapper.cpp:70-109: a row x N tile of
 * vector accumulators, FMAs in CSR order) as SIMD code: 64-column tiles (four 16-float vectors),
 * OpenMP over rows.  N must be a multiple of 64 (returns -1 otherwise).  Bit-identical to
 * orc_csr_spmm. */
int orc_csr_spmm_fast(int64_t M, int64_t N, const int32_t *row_ptrs, const int32_t *col_inds, const float *values,
                      const float *B, int64_t ldb, float *C, int64_t ldc, int num_threads) {
    if (N % 64 != 0) return -1;
#ifdef _OPENMP
    if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(num_threads)
#endif
    for (int64_t i = 0; i < M; ++i) {
        for (int64_t j0 = 0; j0 < N; j0 += 64) {
            v16 c0 = {0}, c1 = {0}, c2 = {0}, c3 = {0};
            for (int32_t p = row_ptrs[i]; p < row_ptrs[i + 1]; ++p) {
                const float a = values[p];
                const float *b = B + (int64_t)col_inds[p] * ldb + j0;
                c0 += a * ld16(b);
                c1 += a * ld16(b + 16);
                c2 += a * ld16(b + 32);
                c3 += a * ld16(b + 48);
            }
            float *o = C + i * ldc + j0;
            st16(o, c0);
            st16(o + 16, c1);
            st16(o + 32, c2);
            st16(o + 48, c3);
        }
    }
    return 0;
}
