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
 * code generator emits one routine per nanokernel.  N_r = 16 floats (four 128-bit vectors per row;
 * 8 floats for M_r > 4); OpenMP threads split the row panels.
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

/* 128-bit vectors: one NEON register on aarch64, one SSE/AVX register on x86-64.  A strip of 16
 * floats is four of them per row (wider generic vectors are lowered through memory). */
typedef float v4 __attribute__((vector_size(16)));

/* Descriptor index of (global panel gp, K tile tj): units are ordered row tile, K tile, panel. */
static int64_t fast_unit(int64_t gp, int64_t tj, int64_t ppt, int64_t T, int64_t P) {
    int64_t ti = gp / ppt, p = gp % ppt;
    int64_t p_lo = ti * ppt;
    int64_t n_in = (p_lo + ppt < P ? ppt : P - p_lo);
    return p_lo * T + tj * n_in + p;
}

static inline v4 ld4(const float *p) {
    v4 v;
    memcpy(&v, p, sizeof v);
    return v;
}
static inline void st4(float *p, v4 v) { memcpy(p, &v, sizeof v); }
static inline v4 relu4(v4 v) { /* fmaxf(o, 0), as the checker's epilogue */
    float t[4];
    memcpy(t, &v, sizeof t);
    for (int j = 0; j < 4; ++j) t[j] = fmaxf(t[j], 0.0f);
    memcpy(&v, t, sizeof t);
    return v;
}
/* acc row r (four vectors) += a * (b0, b1, b2, b3) */
#define FMA_ROW(r, a)          \
    do {                       \
        const float s_ = (a);  \
        r##0 += s_ * b0;       \
        r##1 += s_ * b1;       \
        r##2 += s_ * b2;       \
        r##3 += s_ * b3;       \
    } while (0)

/* One nanokernel group of an M_r <= 4 panel: n entries of pattern P (compile-time constant). */
#define GROUP4(P)                                                  \
    case P:                                                        \
        for (int32_t e = 0; e < n; ++e) {                          \
            const float *bp = B + (int64_t)cols[c++] * ldb + j0;   \
            const v4 b0 = ld4(bp), b1 = ld4(bp + 4), b2 = ld4(bp + 8), b3 = ld4(bp + 12); \
            if ((P) & 1) FMA_ROW(x, vp[v++]);                      \
            if ((P) & 2) FMA_ROW(y, vp[v++]);                      \
            if ((P) & 4) FMA_ROW(z, vp[v++]);                      \
            if ((P) & 8) FMA_ROW(w, vp[v++]);                      \
        }                                                          \
        break;

static void panel_mr4(int num_nkern, const int32_t *id_to_pattern, const uint8_t *arena, const fast_desc *descs,
                      int64_t gp, int64_t M, int64_t P, int64_t ppt, int64_t T, const float *B, int64_t ldb, float *C,
                      int64_t ldc, int64_t N, int load_c, int epilogue, int mr) {
    for (int64_t j0 = 0; j0 + 16 <= N; j0 += 16) {
        const v4 zero = {0, 0, 0, 0};
        v4 x0 = zero, x1 = zero, x2 = zero, x3 = zero, y0 = zero, y1 = zero, y2 = zero, y3 = zero;
        v4 z0 = zero, z1 = zero, z2 = zero, z3 = zero, w0 = zero, w1 = zero, w2 = zero, w3 = zero;
        const int64_t r0 = gp * mr;
        if (load_c) {
#define LOAD_ROW(r, q)                                                                            \
    if (mr > q && r0 + q < M) {                                                                   \
        const float *cp = C + (r0 + q) * ldc + j0;                                                \
        r##0 = ld4(cp); r##1 = ld4(cp + 4); r##2 = ld4(cp + 8); r##3 = ld4(cp + 12);               \
    }
            LOAD_ROW(x, 0) LOAD_ROW(y, 1) LOAD_ROW(z, 2) LOAD_ROW(w, 3)
#undef LOAD_ROW
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
#define STORE_ROW(r, q)                                                                             \
    if (mr > q && r0 + q < M) {                                                                     \
        float *cp = C + (r0 + q) * ldc + j0;                                                        \
        if (epilogue == 1) {                                                                        \
            r##0 = relu4(r##0); r##1 = relu4(r##1); r##2 = relu4(r##2); r##3 = relu4(r##3);         \
        }                                                                                           \
        st4(cp, r##0); st4(cp + 4, r##1); st4(cp + 8, r##2); st4(cp + 12, r##3);                    \
    }
        STORE_ROW(x, 0) STORE_ROW(y, 1) STORE_ROW(z, 2) STORE_ROW(w, 3)
#undef STORE_ROW
    }
}

/* Any M_r <= 8: the rows of each group's pattern in a small list (runtime); used for M_r > 4.
 * Strips of 8 floats (two vectors per row) so that 8 rows of accumulators stay in registers. */
static void panel_generic(int mr, int num_nkern, const int32_t *id_to_pattern, const uint8_t *arena,
                          const fast_desc *descs, int64_t gp, int64_t M, int64_t P, int64_t ppt, int64_t T,
                          const float *B, int64_t ldb, float *C, int64_t ldc, int64_t N, int load_c, int epilogue) {
    for (int64_t j0 = 0; j0 + 8 <= N; j0 += 8) {
        v4 lo[8], hi[8];
        const int64_t r0 = gp * mr;
        for (int r = 0; r < mr; ++r) {
            const v4 z = {0, 0, 0, 0};
            const int ld = load_c && r0 + r < M;
            lo[r] = ld ? ld4(C + (r0 + r) * ldc + j0) : z;
            hi[r] = ld ? ld4(C + (r0 + r) * ldc + j0 + 4) : z;
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
                    const float *bp = B + (int64_t)cols[c++] * ldb + j0;
                    const v4 b0 = ld4(bp), b1 = ld4(bp + 4);
                    for (int q = 0; q < nr; ++q) {
                        const float a = vp[v++];
                        lo[rows[q]] += a * b0;
                        hi[rows[q]] += a * b1;
                    }
                }
            }
        }
        for (int r = 0; r < mr; ++r) {
            if (r0 + r >= M) continue;
            v4 a = lo[r], b = hi[r];
            if (epilogue == 1) {
                a = relu4(a);
                b = relu4(b);
            }
            st4(C + (r0 + r) * ldc + j0, a);
            st4(C + (r0 + r) * ldc + j0 + 4, b);
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
 * vector accumulators, FMAs in CSR order) as SIMD code: 64-column tiles, 32 columns (eight 128-bit
 * vectors) in registers at a time, OpenMP over rows.  N must be a multiple of 64 (returns -1 otherwise).  Bit-identical to
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
            for (int h = 0; h < 64; h += 32) { /* 32 columns (8 vectors) of the 64-column tile at a time */
                const v4 z = {0, 0, 0, 0};
                v4 c0 = z, c1 = z, c2 = z, c3 = z, c4 = z, c5 = z, c6 = z, c7 = z;
                for (int32_t p = row_ptrs[i]; p < row_ptrs[i + 1]; ++p) {
                    const float a = values[p];
                    const float *b = B + (int64_t)col_inds[p] * ldb + j0 + h;
                    c0 += a * ld4(b);
                    c1 += a * ld4(b + 4);
                    c2 += a * ld4(b + 8);
                    c3 += a * ld4(b + 12);
                    c4 += a * ld4(b + 16);
                    c5 += a * ld4(b + 20);
                    c6 += a * ld4(b + 24);
                    c7 += a * ld4(b + 28);
                }
                float *o = C + i * ldc + j0 + h;
                st4(o, c0);
                st4(o + 4, c1);
                st4(o + 8, c2);
                st4(o + 12, c3);
                st4(o + 16, c4);
                st4(o + 20, c5);
                st4(o + 24, c6);
                st4(o + 28, c7);
            }
        }
    }
    return 0;
}
