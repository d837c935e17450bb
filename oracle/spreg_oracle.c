/*
 * spreg_oracle.c -- CPU oracle for the sparse-register-tiling SpMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline / reference arm may load this library, and only as the checker or the timed
 * CPU baseline.  The product (libspreg.so) never calls it.
 *
 * It restates, in plain C, the reference's packer and executor for one sparse weight A:
 *   - pattern code of a panel column .......... sbench/SOP/sop_utils.py:25-30,
 *                                               sbench/SOP/distribution.py:10-15
 *   - mapping a pattern to nanokernel codes .... sbench/SOP/sop_driver.py:50-65
 *   - sort_and_encode_patterns / permute ....... sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:46-98
 *   - SOPTile::pack_panel ...................... template:129-217
 *   - SOPTile::pack_tile arena layout .......... template:219-261
 *   - M_c x K_c tiling, load_c, EMPTY tiles .... cpp_testbed/demo/count_nkerns.cpp:58-128
 *   - executor (per-nanokernel count loops,
 *     ascending-row FMAs, load_c) ............... template:265-305 and
 *                                               tools/codegen/gen_vector_specialized.py:266-357
 *   - CSR baseline (row x N-tile FMAs) ......... sbench/SOP/_C/pytorch_csr_wrapper.cpp:70-191,
 *                                               cpp_testbed/src/spmm/baselines/spmm_csr_c.cpp:67-176
 * The executor calls fmaf() explicitly in packed-entry order, so a GPU kernel that chains
 * fmaf() in the same order per output element matches it bit for bit.  Build with
 * -ffp-contract=off so that no other expression is contracted.
 *
 * Nanokernel id order (absent from the reference: MicroKernel::encode_nkern_pattern lives in
 * the un-vendored spmm-nano-kernels submodule) is the set sorted by (popcount, value), after
 * the popcount sort of tools/codegen/gen_vector_specialized.py:113.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_ZERO 0xFFFF
#define ORC_INVALID (-1)

enum { ORC_F32 = 0, ORC_BF16 = 1, ORC_F16 = 2 };

typedef struct {
    int64_t values_off, cols_off, counts_off;
    int32_t num_values, num_cols;
} orc_desc; /* same layout as spreg_panel_desc */

static int popc(uint32_t x) { return __builtin_popcount(x); }
static int64_t align64(int64_t x) { return (x + 63) & ~(int64_t)63; }

/* ------------------------------------------------------------ IEEE conversions */
static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* float -> bfloat16, round to nearest even (NaN -> quiet NaN with the sign kept). */
uint16_t orc_f32_to_bf16(float f) {
    uint32_t u = f2u(f);
    if ((u & 0x7FFFFFFFu) > 0x7F800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
float orc_bf16_to_f32(uint16_t h) { return u2f((uint32_t)h << 16); }

/* float -> IEEE binary16, round to nearest even, from the format definition. */
uint16_t orc_f32_to_f16(float f) {
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) /* inf / nan */
        return (uint16_t)(sign | 0x7C00u | (ax > 0x7F800000u ? (0x200u | ((ax >> 13) & 0x3FFu)) : 0u));
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u); /* >= 65520 rounds to inf */
    if (ax >= 0x38800000u) {                                  /* normal binary16 (>= 2^-14) */
        uint32_t mant = ax & 0x7FFFFFu;
        uint32_t e = (ax >> 23) - 127u + 15u;
        uint32_t h = (e << 10) | (mant >> 13);
        uint32_t rem = mant & 0x1FFFu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    if (ax < 0x33000000u) return (uint16_t)sign; /* below 2^-25: rounds to zero */
    {                                            /* subnormal binary16, unit 2^-24 */
        uint32_t mant = (ax & 0x7FFFFFu) | 0x800000u;
        int e = (int)(ax >> 23);
        int shift = 126 - e;
        uint32_t h = mant >> shift;
        uint32_t rem = mant & ((1u << shift) - 1u);
        uint32_t halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
}
float orc_f16_to_f32(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = ((uint32_t)h >> 10) & 0x1Fu;
    uint32_t m = (uint32_t)h & 0x3FFu;
    if (e == 0x1Fu) return u2f(sign | 0x7F800000u | (m << 13));
    if (e == 0) {
        if (m == 0) return u2f(sign);
        float v = (float)m * (1.0f / 16777216.0f); /* m * 2^-24, exact */
        return sign ? -v : v;
    }
    return u2f(sign | ((e - 15u + 127u) << 23) | (m << 13));
}

void orc_f32_to_bf16_array(const float *in, uint16_t *out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = orc_f32_to_bf16(in[i]);
}
void orc_f32_to_f16_array(const float *in, uint16_t *out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = orc_f32_to_f16(in[i]);
}

static float load_as_f32(const void *p, int64_t i, int dtype) {
    if (dtype == ORC_F32) return ((const float *)p)[i];
    if (dtype == ORC_BF16) return orc_bf16_to_f32(((const uint16_t *)p)[i]);
    return orc_f16_to_f32(((const uint16_t *)p)[i]);
}
static void store_from_f32(void *p, int64_t i, int dtype, float v) {
    if (dtype == ORC_F32) ((float *)p)[i] = v;
    else if (dtype == ORC_BF16) ((uint16_t *)p)[i] = orc_f32_to_bf16(v);
    else ((uint16_t *)p)[i] = orc_f32_to_f16(v);
}
static int dtype_bytes(int dtype) { return dtype == ORC_F32 ? 4 : 2; }

/* Power-of-two scale of an F16 row panel: 2^e with max|v| = m * 2^e, m in [0.5, 1). */
float orc_f16_panel_scale(float maxabs) {
    int e = 0;
    if (!(maxabs > 0.0f) || !isfinite(maxabs)) return 1.0f;
    frexpf(maxabs, &e);
    return ldexpf(1.0f, e);
}

/* ------------------------------------------------------------- nanokernel set
 * Builds id <-> pattern tables.  nanokernels == NULL: the set is every distinct nonzero
 * code the mapping lists.  Returns the number of nanokernels or -1 on a bad pattern. */
int orc_mapping_build(int mr, const int32_t *map_offsets, const int32_t *map_codes, const int32_t *nanokernels,
                      int num_nanokernels, int32_t *id_to_pattern, int32_t *code_to_id) {
    int np = 1 << mr;
    unsigned char present[256];
    memset(present, 0, sizeof present);
    if (mr < 1 || mr > 8) return -1;
    if (nanokernels) {
        for (int i = 0; i < num_nanokernels; ++i) {
            int p = nanokernels[i];
            if (p <= 0 || p >= np) return -1;
            present[p] = 1;
        }
    } else {
        for (int p = 0; p < np; ++p)
            for (int32_t q = map_offsets[p]; q < map_offsets[p + 1]; ++q) {
                int c = map_codes[q];
                if (c < 0 || c >= np) return -1;
                if (c) present[c] = 1;
            }
    }
    int n = 0;
    for (int pc = 1; pc <= mr; ++pc)
        for (int p = 1; p < np; ++p)
            if (present[p] && popc((uint32_t)p) == pc) id_to_pattern[n++] = p;
    for (int c = 0; c < 256; ++c) code_to_id[c] = ORC_INVALID;
    code_to_id[0] = ORC_ZERO;
    for (int id = 0; id < n; ++id) code_to_id[id_to_pattern[id]] = id;
    return n;
}

/* Pattern codes of one panel (sop_utils.py:25-30 on the transposed panel, sop_driver.py:69):
 * bit r of codes[c] is set iff A[row0 + r][c] != 0; rows >= M read as zero. */
void orc_panel_patterns(const float *A, int64_t M, int64_t lda, int mr, int64_t row0, int64_t c_lo, int64_t c_hi,
                        int32_t *codes) {
    for (int64_t c = c_lo; c < c_hi; ++c) {
        int32_t code = 0;
        for (int r = 0; r < mr; ++r)
            if (row0 + r < M && A[(row0 + r) * lda + c] != 0.0f) code |= 1 << r;
        codes[c - c_lo] = code;
    }
}

/* ---------------------------------------------------------- sort_and_encode
 * Comparator of template:76-78: a before b iff id(a) != ZERO and (id(b) == ZERO or id(a) < id(b)),
 * applied by a stable merge sort (std::stable_sort semantics). */
static int enc_less(int32_t a, int32_t b) { return (b == ORC_ZERO || a < b) && (a != ORC_ZERO); }

static void merge_sort_idx(int32_t *idx, int32_t *tmp, int64_t n, const int32_t *key) {
    for (int64_t w = 1; w < n; w *= 2) {
        for (int64_t lo = 0; lo < n; lo += 2 * w) {
            int64_t mid = lo + w < n ? lo + w : n;
            int64_t hi = lo + 2 * w < n ? lo + 2 * w : n;
            int64_t i = lo, j = mid, o = lo;
            while (i < mid && j < hi) {
                if (enc_less(key[idx[j]], key[idx[i]])) tmp[o++] = idx[j++];
                else tmp[o++] = idx[i++];
            }
            while (i < mid) tmp[o++] = idx[i++];
            while (j < hi) tmp[o++] = idx[j++];
        }
        memcpy(idx, tmp, (size_t)n * sizeof(int32_t));
    }
}

/* In-place permutation of template:46-68 (cycle following).  Result: v_new[i] = v_old[order[i]]. */
void orc_permute_inplace(const int32_t *order, int32_t *v, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        int64_t s = order[i];
        while (s < i) s = order[s];
        int32_t t = v[i];
        v[i] = v[s];
        v[s] = t;
    }
}

/* sort_and_encode_patterns (template:84-98).  Returns 0, or -1 if a code is not a nanokernel. */
int orc_sort_and_encode(const int32_t *code_to_id, const int32_t *pat_codes, int64_t n, int32_t *encoded,
                        int32_t *order) {
    int32_t *tmp = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) {
        int32_t c = pat_codes[i];
        if (c < 0 || c > 255 || code_to_id[c] == ORC_INVALID) { free(tmp); return -1; }
        encoded[i] = code_to_id[c];
        order[i] = (int32_t)i;
    }
    merge_sort_idx(order, tmp, n, encoded);
    orc_permute_inplace(order, encoded, n);
    free(tmp);
    return 0;
}

/* ---------------------------------------------------------------- pack_panel
 * SOPTile::pack_panel (template:129-217).  dense_panel is (panel_cols x mr): dense_panel[c*mr + r].
 * Outputs counts[num_nkern], cols_out[<= n], values_out[<= n*mr] (as float).
 * Returns 0, -1 bad code, -2 column out of range, -3 invariant num_nnz == padding + nnz failed. */
int orc_pack_panel(int mr, int num_nkern, const int32_t *code_to_id, const int32_t *id_to_pattern, int64_t col_offset,
                   const int32_t *pat_codes, const int32_t *col_indices, int64_t n, const float *dense_panel,
                   int64_t panel_cols, int32_t *counts, int32_t *cols_out, float *values_out, int64_t *num_values,
                   int64_t *num_cols, int64_t *padding) {
    int32_t *enc = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    int32_t *order = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    int32_t *cols = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    int rc = 0;
    if (orc_sort_and_encode(code_to_id, pat_codes, n, enc, order)) { rc = -1; goto done; }
    memcpy(cols, col_indices, (size_t)n * sizeof(int32_t));
    orc_permute_inplace(order, cols, n);
    int64_t start_zero = n;
    for (int64_t p = 0; p < n; ++p)
        if (enc[p] == ORC_ZERO) { start_zero = p; break; }
    for (int id = 0; id < num_nkern; ++id) counts[id] = 0;
    int64_t vo = 0, u = 0, pad = 0;
    for (int64_t p = 0; p < start_zero; ++p) {
        int32_t e = enc[p];
        int32_t col = cols[p];
        if (col < 0 || col >= panel_cols) { rc = -2; goto done; }
        counts[e]++;
        cols_out[u++] = (int32_t)(col + col_offset);
        uint32_t pat = (uint32_t)id_to_pattern[e];
        int row = 0;
        while (pat) {
            if (pat & 1u) {
                float v = dense_panel[(int64_t)col * mr + row];
                if (v == 0.0f) pad++;
                values_out[vo++] = v;
            }
            pat >>= 1;
            row++;
        }
    }
    int64_t nnz = 0;
    for (int64_t i = 0; i < panel_cols * mr; ++i) nnz += dense_panel[i] != 0.0f;
    *num_values = vo;
    *num_cols = u;
    *padding = pad;
    if (vo != pad + nnz) rc = -3;
done:
    free(enc);
    free(order);
    free(cols);
    return rc;
}

/* ---------------------------------------------------------------- pack_dense
 * Whole matrix: panels of mr rows (rows padded with zeros to a multiple of mr), tiles of
 * m_tile x k_tile (0 = whole extent) visited row tile, K tile, panel (count_nkerns.cpp:78-125);
 * per unit, codes come from the mapping applied to every column in ascending order
 * (sop_driver.py:50-65) and pack_panel emits them; units are laid out as pack_tile lays out
 * panels (template:219-261).  value_dtype F16 divides values by a per-row-panel power-of-two
 * scale before rounding.  With arena == NULL only the sizes are computed.
 *
 * out_sizes[0..9] = num_units, arena_bytes, num_values, num_col_indices, padding, nnz,
 *                   required_storage, empty_units, num_k_tiles, panels_per_tile.
 * Returns 0 or the first pack_panel error. */
int orc_pack_dense(int mr, int num_nkern, const int32_t *code_to_id, const int32_t *id_to_pattern,
                   const int32_t *map_offsets, const int32_t *map_codes, const float *A, int64_t M, int64_t K,
                   int64_t lda, int32_t m_tile, int32_t k_tile, int64_t col_offset, int value_dtype, uint8_t *arena,
                   orc_desc *descs, float *scales, int64_t *out_sizes) {
    int64_t P = (M + mr - 1) / mr;
    int64_t ppt = m_tile > 0 ? m_tile / mr : (P > 0 ? P : 1);
    if (ppt <= 0) ppt = 1;
    int64_t RT = P > 0 ? (P + ppt - 1) / ppt : 0;
    int64_t kt = k_tile > 0 ? k_tile : (K > 0 ? K : 1);
    int64_t T = K > 0 ? (K + kt - 1) / kt : 1;
    int vb = dtype_bytes(value_dtype);

    int64_t maxc = kt;
    int32_t *pcodes = (int32_t *)malloc((size_t)(maxc > 0 ? maxc : 1) * sizeof(int32_t));
    int32_t *ecodes = (int32_t *)malloc((size_t)(maxc * mr + 1) * sizeof(int32_t));
    int32_t *ecols = (int32_t *)malloc((size_t)(maxc * mr + 1) * sizeof(int32_t));
    float *dense = (float *)malloc((size_t)(maxc * mr + 1) * sizeof(float));
    int32_t *counts = (int32_t *)malloc((size_t)(num_nkern + 1) * sizeof(int32_t));
    int32_t *cols_out = (int32_t *)malloc((size_t)(maxc * mr + 1) * sizeof(int32_t));
    float *vals_out = (float *)malloc((size_t)(maxc * mr * mr + 1) * sizeof(float));

    /* per-row-panel scale for F16 */
    if (value_dtype == ORC_F16 && scales) {
        for (int64_t gp = 0; gp < P; ++gp) {
            float mx = 0.0f;
            for (int r = 0; r < mr; ++r) {
                int64_t row = gp * mr + r;
                if (row >= M) break;
                for (int64_t c = 0; c < K; ++c) {
                    float a = fabsf(A[row * lda + c]);
                    if (a > mx) mx = a;
                }
            }
            scales[gp] = orc_f16_panel_scale(mx);
        }
    }

    int64_t unit = 0, off = 0, tot_v = 0, tot_u = 0, tot_pad = 0, tot_nnz = 0, req = 0, empty = 0;
    int rc = 0;
    for (int64_t ti = 0; ti < RT; ++ti) {
        int64_t p_lo = ti * ppt, p_hi = p_lo + ppt < P ? p_lo + ppt : P;
        for (int64_t tj = 0; tj < T; ++tj) {
            int64_t c_lo = tj * kt, c_hi = c_lo + kt < K ? c_lo + kt : K;
            int64_t ncols = c_hi > c_lo ? c_hi - c_lo : 0;
            int64_t tile_nnz = 0;
            int64_t first_unit = unit;
            for (int64_t gp = p_lo; gp < p_hi; ++gp, ++unit) {
                orc_panel_patterns(A, M, lda, mr, gp * mr, c_lo, c_hi, pcodes);
                int64_t n = 0;
                for (int64_t c = 0; c < ncols; ++c) {
                    int32_t p = pcodes[c];
                    for (int32_t q = map_offsets[p]; q < map_offsets[p + 1]; ++q) {
                        ecodes[n] = map_codes[q];
                        ecols[n] = (int32_t)c;
                        n++;
                    }
                    for (int r = 0; r < mr; ++r) {
                        int64_t row = gp * mr + r;
                        dense[c * mr + r] = row < M ? A[row * lda + c_lo + c] : 0.0f;
                    }
                }
                int64_t nv = 0, nu = 0, pad = 0;
                int prc = orc_pack_panel(mr, num_nkern, code_to_id, id_to_pattern, col_offset + c_lo, ecodes, ecols, n,
                                         dense, ncols, counts, cols_out, vals_out, &nv, &nu, &pad);
                if (prc && !rc) rc = prc;
                int64_t nnz = 0;
                for (int64_t i = 0; i < ncols * mr; ++i) nnz += dense[i] != 0.0f;
                tile_nnz += nnz;
                int64_t voff = off, coff = off + align64(nv * vb), koff = coff + align64(nu * 4);
                int64_t next = koff + align64((int64_t)num_nkern * 4);
                if (arena) {
                    memset(arena + off, 0, (size_t)(next - off));
                    float s = (value_dtype == ORC_F16 && scales) ? scales[gp] : 1.0f;
                    float inv = 1.0f / s; /* exact: s is a power of two */
                    for (int64_t i = 0; i < nv; ++i) {
                        float v = vals_out[i];
                        if (value_dtype == ORC_F16) v = v * inv;
                        store_from_f32(arena + voff, i, value_dtype, v);
                    }
                    memcpy(arena + coff, cols_out, (size_t)nu * 4);
                    memcpy(arena + koff, counts, (size_t)num_nkern * 4);
                    descs[unit].values_off = voff;
                    descs[unit].cols_off = coff;
                    descs[unit].counts_off = koff;
                    descs[unit].num_values = (int32_t)nv;
                    descs[unit].num_cols = (int32_t)nu;
                }
                off = next;
                tot_v += nv;
                tot_u += nu;
                tot_pad += pad;
                tot_nnz += nnz;
                req += nv * vb + nu * 4 + (int64_t)num_nkern * 4 + 3 * 64;
            }
            if (tile_nnz == 0) empty += unit - first_unit;
        }
    }
    out_sizes[0] = unit;
    out_sizes[1] = off;
    out_sizes[2] = tot_v;
    out_sizes[3] = tot_u;
    out_sizes[4] = tot_pad;
    out_sizes[5] = tot_nnz;
    out_sizes[6] = req;
    out_sizes[7] = empty;
    out_sizes[8] = T;
    out_sizes[9] = ppt;
    free(pcodes);
    free(ecodes);
    free(ecols);
    free(dense);
    free(counts);
    free(cols_out);
    free(vals_out);
    return rc;
}

/* Descriptor index of (global panel gp, K tile tj): units are ordered row tile, K tile, panel. */
static int64_t unit_index(int64_t gp, int64_t tj, int64_t ppt, int64_t T, int64_t P) {
    int64_t ti = gp / ppt, p = gp % ppt;
    int64_t p_lo = ti * ppt;
    int64_t n_in = (p_lo + ppt < P ? ppt : P - p_lo);
    return p_lo * T + tj * n_in + p;
}

/* ------------------------------------------------------------------ executor
 * sop_multiple_panel_executor (template:265-305) with the microkernel semantics of
 * tools/codegen/gen_vector_specialized.py:266-357: per row panel, accumulators start at C
 * (load_c) or zero; for every nanokernel id in order, for count entries, B row = col index,
 * and for each set row of the id's pattern in ascending order acc[row] += value * B[row].
 * K tiles of one row panel run in order and keep accumulating (load_c of tiles tj > 0,
 * count_nkerns.cpp:93).  F16 values: acc starts at zero and C = acc * scale (+ C if load_c).
 * Columns are processed in strips of `strip` floats.  Threads split row panels. */
void orc_execute(int mr, int num_nkern, const int32_t *id_to_pattern, const uint8_t *arena, const orc_desc *descs,
                 const float *scales, int value_dtype, int64_t M, int64_t P, int64_t ppt, int64_t T, const void *B,
                 int b_dtype, int64_t ldb, void *C, int c_dtype, int64_t ldc, int64_t N, int load_c, int epilogue,
                 int num_threads) {
    const int STRIP = 16;
    const int scaled = value_dtype == ORC_F16;
#ifdef _OPENMP
    if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(num_threads)
#endif
    for (int64_t gp = 0; gp < P; ++gp) {
        float acc[8][16];
        for (int64_t j0 = 0; j0 < N; j0 += STRIP) {
            int64_t w = N - j0 < STRIP ? N - j0 : STRIP;
            for (int r = 0; r < mr; ++r) {
                int64_t row = gp * mr + r;
                for (int64_t j = 0; j < w; ++j)
                    acc[r][j] = (!scaled && load_c && row < M) ? load_as_f32(C, row * ldc + j0 + j, c_dtype) : 0.0f;
            }
            for (int64_t tj = 0; tj < T; ++tj) {
                const orc_desc *d = &descs[unit_index(gp, tj, ppt, T, P)];
                const int32_t *cnt = (const int32_t *)(arena + d->counts_off);
                const int32_t *cols = (const int32_t *)(arena + d->cols_off);
                const uint8_t *vals = arena + d->values_off;
                int64_t c = 0, v = 0;
                /* FP32 values and B over a whole strip: the same fmaf chain per element, with fixed-length
                 * inner loops the compiler turns into vector FMAs (the reference's executor is SIMD too) */
                const int fast = b_dtype == ORC_F32 && value_dtype == ORC_F32 && w == STRIP;
                for (int id = 0; fast && id < num_nkern; ++id) {
                    const int32_t n = cnt[id];
                    const uint32_t pat = (uint32_t)id_to_pattern[id];
                    const float *vp = (const float *)vals;
                    for (int32_t e = 0; e < n; ++e, ++c) {
                        const float *bp = (const float *)B + cols[c] * ldb + j0;
                        for (int r = 0; r < mr; ++r) {
                            if (!((pat >> r) & 1u)) continue;
                            const float a = vp[v++];
                            for (int j = 0; j < 16; ++j) acc[r][j] = fmaf(a, bp[j], acc[r][j]);
                        }
                    }
                }
                for (int id = 0; !fast && id < num_nkern; ++id) {
                    int32_t n = cnt[id];
                    uint32_t pat = (uint32_t)id_to_pattern[id];
                    for (int32_t e = 0; e < n; ++e, ++c) {
                        int64_t k = cols[c];
                        float b[16];
                        for (int64_t j = 0; j < w; ++j) b[j] = load_as_f32(B, k * ldb + j0 + j, b_dtype);
                        for (int r = 0; r < mr; ++r) {
                            if (!((pat >> r) & 1u)) continue;
                            float a = load_as_f32(vals, v++, value_dtype);
                            for (int64_t j = 0; j < w; ++j) acc[r][j] = fmaf(a, b[j], acc[r][j]);
                        }
                    }
                }
            }
            for (int r = 0; r < mr; ++r) {
                int64_t row = gp * mr + r;
                if (row >= M) continue;
                for (int64_t j = 0; j < w; ++j) {
                    float o = acc[r][j];
                    if (scaled) {
                        float s = scales[gp];
                        o = load_c ? fmaf(o, s, load_as_f32(C, row * ldc + j0 + j, c_dtype)) : o * s;
                    }
                    if (epilogue == 1) o = fmaxf(o, 0.0f);
                    store_from_f32(C, row * ldc + j0 + j, c_dtype, o);
                }
            }
        }
    }
}

/* ---------------------------------------------------------------- CSR baseline
 * Row x N-tile CSR SpMM (pytorch_csr_wrapper.cpp:70-109, _dispatch_n_tile_size :140-191),
 * OpenMP dynamic over rows (spmm_csr_c.cpp:104): C[i, j:j+nt] = sum_p val[p] * B[col[p], j:j+nt]
 * with FMAs in CSR order; the N tail is handled elementwise. */
void orc_csr_spmm(int64_t M, int64_t N, const int32_t *row_ptrs, const int32_t *col_inds, const float *values,
                  const float *B, int64_t ldb, float *C, int64_t ldc, int num_threads) {
    const int NT = 64;
#ifdef _OPENMP
    if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(num_threads)
#endif
    for (int64_t i = 0; i < M; ++i) {
        float acc[64];
        for (int64_t j0 = 0; j0 < N; j0 += NT) {
            int64_t w = N - j0 < NT ? N - j0 : NT;
            for (int64_t j = 0; j < w; ++j) acc[j] = 0.0f;
            if (w == NT) { /* whole tile: fixed-length loop, vectorised by the compiler */
                for (int32_t p = row_ptrs[i]; p < row_ptrs[i + 1]; ++p) {
                    const float a = values[p];
                    const float *b = B + (int64_t)col_inds[p] * ldb + j0;
                    for (int j = 0; j < NT; ++j) acc[j] = fmaf(a, b[j], acc[j]);
                }
            } else {
                for (int32_t p = row_ptrs[i]; p < row_ptrs[i + 1]; ++p) {
                    float a = values[p];
                    const float *b = B + (int64_t)col_inds[p] * ldb + j0;
                    for (int64_t j = 0; j < w; ++j) acc[j] = fmaf(a, b[j], acc[j]);
                }
            }
            for (int64_t j = 0; j < w; ++j) C[i * ldc + j0 + j] = acc[j];
        }
    }
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
