// capi.cu -- extern "C" entry points of libspreg.so (declared in include/spreg.h).
#include "spreg_common.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace spreg {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

// Implemented in pack.cu / exec.cu.
int dense_rows_bf16_impl(const void *, int64_t, int64_t, int64_t, const int32_t *, const void *, int64_t, void *,
                         int64_t, int64_t, int32_t, int32_t, int32_t, cudaStream_t);
int dense_rows_batched_impl(const spreg_dense_rows_item *, int32_t, cudaStream_t);
int dense_rows_f32_batched_impl(const spreg_dense_rows_f32_item *, int32_t, cudaStream_t);
int split_rows_f32_impl(const float *, int64_t, int64_t, int64_t, void *, int64_t, float *, cudaStream_t);
int tc_plan_create_f32_impl(const spreg_dense_rows_f32_item *, int32_t, void **, cudaStream_t);
int tc_plan_create_bf16_impl(const spreg_dense_rows_item *, int32_t, void **, cudaStream_t);
int tc_plan_run_impl(const void *, cudaStream_t);
void tc_plan_destroy_impl(void *);
int pack_from_arena_impl(const spreg_mapping *, const spreg_arena_geom *, const void *, int64_t,
                         const spreg_panel_desc *, int64_t, const float *, int64_t, spreg_packed **, cudaStream_t);
int pack_dense_impl(const spreg_mapping *, const float *, int64_t, int64_t, int64_t, const spreg_pack_opts *,
                    spreg_packed **, cudaStream_t);
int pack_csr_impl(const spreg_mapping *, const spreg_csr *, const spreg_pack_opts *, spreg_packed **, cudaStream_t);
int pack_lists_impl(const spreg_mapping *, int64_t, int64_t, int64_t, const std::vector<int32_t> &,
                    const std::vector<int32_t> &, const std::vector<int64_t> &, const std::vector<float> &,
                    const std::vector<int64_t> &, const std::vector<int64_t> &, const std::vector<int64_t> &, int,
                    spreg_packed **, cudaStream_t);
int sort_encode_impl(const spreg_mapping *, const int32_t *, int64_t, int32_t *, int32_t *, cudaStream_t);
void packed_release(spreg_packed *);
int execute_impl(const spreg_packed *, const spreg_exec_args *, cudaStream_t);
int execute_timed_impl(const spreg_packed *, const spreg_exec_args *, int64_t, double *, cudaStream_t);
int execute_batched_impl(const spreg_work_item *, int32_t, cudaStream_t);
int load_balance_plan_impl(const spreg_packed *, const spreg_exec_args *, int64_t *, int32_t *, int32_t *, int64_t);
int explain_impl(const spreg_packed *, const spreg_exec_args *, char *, int64_t);
int device_status_impl(int32_t *, int);
int selftest_wait_impl(uint32_t, int32_t *, uint32_t *, cudaStream_t);
int csr_spmm_impl(int64_t, int64_t, int64_t, int64_t, const int32_t *, const int32_t *, const float *, const float *,
                  int64_t, float *, int64_t, int32_t, cudaStream_t);
int csr_spmm_timed_impl(int64_t, int64_t, int64_t, int64_t, const int32_t *, const int32_t *, const float *,
                        const float *, int64_t, float *, int64_t, int32_t, int64_t, double *, cudaStream_t);

static std::mutex g_map_mu;

const MapTable *mapping_device_table(const spreg_mapping *m, int *status) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        *status = SPREG_ERR_CUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_map_mu);
    spreg_mapping *mm = const_cast<spreg_mapping *>(m);
    if (!mm->dev[dev]) {
        void *p = nullptr;
        e = cudaMalloc(&p, sizeof(MapTable));
        if (e == cudaSuccess) e = cudaMemcpy(p, &mm->host, sizeof(MapTable), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (p) cudaFree(p);
            set_error(std::string("mapping upload: ") + cudaGetErrorString(e));
            *status = SPREG_ERR_CUDA;
            return nullptr;
        }
        mm->dev[dev] = p;
    }
    *status = SPREG_OK;
    return reinterpret_cast<const MapTable *>(mm->dev[dev]);
}

}  // namespace spreg

using namespace spreg;

// ====================================================================== SOPTile staging
struct spreg_tile {
    const spreg_mapping *map = nullptr;
    int64_t rows = 0, cols = 0, num_panels = 0;
    std::vector<char> packed_flag;
    // per panel staged data
    std::vector<std::vector<int32_t>> codes, colidx;
    std::vector<std::vector<float>> dense;
    std::vector<int64_t> panel_cols, col_offset;
    spreg_packed *packed = nullptr;
};

// ====================================================================== MatMulSpecialized
struct spreg_matmul {
    int32_t m = 0, k = 0, n = 0;
    spreg_tile_config cfg = {};
    spreg_packed *packed = nullptr;
    cudaStream_t stream = nullptr;
    float *dB = nullptr, *dC = nullptr;
    int32_t alloc_n = 0;
    int32_t direct_output = 1;  // store C straight into mapped page-locked host C (no copy out)
};

// True when p is page-locked host memory that the device addresses at the same pointer.
static bool host_mapped(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // not memory CUDA knows: clear the (non-sticky) error it reported
        return false;
    }
    return at.type == cudaMemoryTypeHost && at.devicePointer == p;
}

extern "C" {

const char *spreg_last_error(void) { return g_last_error.c_str(); }

int spreg_version(void) { return 200; /* 0.2.0 */ }

// ---------------------------------------------------------------------- mapping
int spreg_mapping_create(int32_t mr, const int32_t *map_offsets, const int32_t *map_codes, const int32_t *nanokernels,
                         int32_t num_nanokernels, spreg_mapping **out) {
    clear_error();
    SPREG_CHECK_ARG(out, "null output");
    *out = nullptr;
    SPREG_CHECK_ARG(mr == 2 || mr == 4 || mr == 6 || mr == 8, "M_r must be 2, 4, 6 or 8 (got %d)", mr);
    SPREG_CHECK_ARG(map_offsets && (map_codes || map_offsets[1 << mr] == 0), "null mapping arrays");
    const int np = 1 << mr;
    SPREG_CHECK_ARG(map_offsets[0] == 0, "map_offsets[0] must be 0");
    for (int p = 0; p < np; ++p)
        SPREG_CHECK_ARG(map_offsets[p + 1] >= map_offsets[p], "map_offsets must be non-decreasing");
    bool present[256] = {};
    if (nanokernels) {
        SPREG_CHECK_ARG(num_nanokernels >= 0 && num_nanokernels <= 255, "bad nanokernel count");
        for (int i = 0; i < num_nanokernels; ++i) {
            const int p = nanokernels[i];
            SPREG_CHECK_ARG(p > 0 && p < np, "nanokernel pattern %d outside [1, 2^M_r)", p);
            present[p] = true;
        }
    }
    for (int p = 0; p < np; ++p) {
        int nz = 0;
        for (int q = map_offsets[p]; q < map_offsets[p + 1]; ++q) {
            const int c = map_codes[q];
            SPREG_CHECK_ARG(c >= 0 && c < np, "pattern %d maps to code %d outside [0, 2^M_r)", p, c);
            if (!c) continue;
            ++nz;
            if (nanokernels) SPREG_CHECK_ARG(present[c], "pattern %d maps to %d, which is not a nanokernel of the module", p, c);
            else present[c] = true;
        }
        if (nz > kMaxCodesPerPattern)
            SPREG_FAIL(SPREG_ERR_UNSUPPORTED, "pattern %d maps to %d nanokernels (at most %d)", p, nz, kMaxCodesPerPattern);
    }
    spreg_mapping *m = new (std::nothrow) spreg_mapping();
    if (!m) SPREG_FAIL(SPREG_ERR_NOMEM, "out of host memory");
    m->mr = mr;
    int n = 0;
    for (int pc = 1; pc <= mr; ++pc)
        for (int p = 1; p < np; ++p)
            if (present[p] && __builtin_popcount(p) == pc) m->id_to_pattern[n++] = p;
    m->num_nkern = n;
    for (int c = 0; c < 256; ++c) m->code_to_id[c] = -1;
    m->code_to_id[0] = SPREG_ZERO_PATTERN_ID;
    for (int id = 0; id < n; ++id) m->code_to_id[m->id_to_pattern[id]] = id;
    MapTable &t = m->host;
    std::memset(&t, 0, sizeof t);
    t.mr = mr;
    t.num_nkern = n;
    for (int c = 0; c < 256; ++c) t.code_to_id[c] = kCodeInvalid;
    t.code_to_id[0] = kCodeZero;
    for (int id = 0; id < n; ++id) {
        t.id_to_pattern[id] = (uint8_t)m->id_to_pattern[id];
        t.code_to_id[m->id_to_pattern[id]] = (uint16_t)id;
    }
    for (int p = 0; p < np; ++p) {
        int k = 0;
        for (int q = map_offsets[p]; q < map_offsets[p + 1]; ++q)
            if (map_codes[q]) t.map_codes[p][k++] = (uint8_t)map_codes[q];
        t.map_n[p] = (uint8_t)k;
    }
    *out = m;
    return SPREG_OK;
}

void spreg_mapping_destroy(spreg_mapping *m) {
    if (!m) return;
    int cur = -1;
    cudaGetDevice(&cur);
    for (int d = 0; d < 64; ++d)
        if (m->dev[d]) {
            cudaSetDevice(d);
            cudaFree(m->dev[d]);
        }
    if (cur >= 0) cudaSetDevice(cur);
    delete m;
}

int32_t spreg_mapping_mr(const spreg_mapping *m) { return m ? m->mr : -1; }
int32_t spreg_mapping_num_nkern(const spreg_mapping *m) { return m ? m->num_nkern : -1; }

int spreg_mapping_nkern_patterns(const spreg_mapping *m, int32_t *out) {
    clear_error();
    SPREG_CHECK_ARG(m && out, "null argument");
    for (int i = 0; i < m->num_nkern; ++i) out[i] = m->id_to_pattern[i];
    return SPREG_OK;
}

int32_t spreg_mapping_encode(const spreg_mapping *m, int32_t pattern) {
    if (!m || pattern < 0 || pattern > 255) return -1;
    return m->code_to_id[pattern];
}

int spreg_sort_and_encode_patterns(const spreg_mapping *m, const int32_t *pat_codes, int64_t n, int32_t *encoded,
                                   int32_t *order, spreg_stream_t stream) {
    clear_error();
    return sort_encode_impl(m, pat_codes, n, encoded, order, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------- packing
int spreg_pack_csr(const spreg_mapping *m, const spreg_csr *a, const spreg_pack_opts *opts, spreg_packed **out,
                   spreg_stream_t stream) {
    clear_error();
    if (out) *out = nullptr;
    return pack_csr_impl(m, a, opts, out, (cudaStream_t)stream);
}

int spreg_pack_dense(const spreg_mapping *m, const float *a, int64_t rows, int64_t cols, int64_t lda,
                     const spreg_pack_opts *opts, spreg_packed **out, spreg_stream_t stream) {
    clear_error();
    if (out) *out = nullptr;
    return pack_dense_impl(m, a, rows, cols, lda, opts, out, (cudaStream_t)stream);
}

int spreg_pack_from_arena(const spreg_mapping *m, const spreg_arena_geom *geom, const void *arena_host,
                          int64_t arena_bytes, const spreg_panel_desc *descs_host, int64_t num_units,
                          const float *scales_host, int64_t num_scales, spreg_packed **out, spreg_stream_t stream) {
    clear_error();
    if (out) *out = nullptr;
    return pack_from_arena_impl(m, geom, arena_host, arena_bytes, descs_host, num_units, scales_host, num_scales, out,
                                (cudaStream_t)stream);
}

int spreg_dense_rows_bf16(const void *a_rows, int64_t rows, int64_t k, int64_t lda, const int32_t *row_index,
                          const void *b, int64_t ldb, void *c, int64_t ldc, int64_t n, int32_t c_dtype,
                          int32_t load_c, int32_t epilogue, spreg_stream_t stream) {
    clear_error();
    return dense_rows_bf16_impl(a_rows, rows, k, lda, row_index, b, ldb, c, ldc, n, c_dtype, load_c, epilogue,
                                (cudaStream_t)stream);
}

int spreg_dense_rows_bf16_batched(const spreg_dense_rows_item *items, int32_t num_items, spreg_stream_t stream) {
    clear_error();
    return dense_rows_batched_impl(items, num_items, (cudaStream_t)stream);
}

int spreg_dense_rows_f32_split(const float *a_rows, int64_t rows, int64_t k, int64_t lda, void *a_split,
                               int64_t ld_split, float *row_scale, spreg_stream_t stream) {
    clear_error();
    return split_rows_f32_impl(a_rows, rows, k, lda, a_split, ld_split, row_scale, (cudaStream_t)stream);
}

int spreg_dense_rows_f32(const spreg_dense_rows_f32_item *item, spreg_stream_t stream) {
    clear_error();
    SPREG_CHECK_ARG(item, "null item");
    return dense_rows_f32_batched_impl(item, 1, (cudaStream_t)stream);
}

int spreg_dense_rows_f32_batched(const spreg_dense_rows_f32_item *items, int32_t num_items, spreg_stream_t stream) {
    clear_error();
    return dense_rows_f32_batched_impl(items, num_items, (cudaStream_t)stream);
}

int spreg_dense_rows_f32_plan_create(const spreg_dense_rows_f32_item *items, int32_t num_items,
                                     spreg_dense_rows_plan **out, spreg_stream_t stream) {
    clear_error();
    return tc_plan_create_f32_impl(items, num_items, reinterpret_cast<void **>(out), (cudaStream_t)stream);
}

int spreg_dense_rows_bf16_plan_create(const spreg_dense_rows_item *items, int32_t num_items,
                                      spreg_dense_rows_plan **out, spreg_stream_t stream) {
    clear_error();
    return tc_plan_create_bf16_impl(items, num_items, reinterpret_cast<void **>(out), (cudaStream_t)stream);
}

int spreg_dense_rows_plan_run(const spreg_dense_rows_plan *plan, spreg_stream_t stream) {
    clear_error();
    return tc_plan_run_impl(plan, (cudaStream_t)stream);
}

void spreg_dense_rows_plan_destroy(spreg_dense_rows_plan *plan) { tc_plan_destroy_impl(plan); }

void spreg_packed_destroy(spreg_packed *p) { packed_release(p); }

int spreg_packed_get_info(const spreg_packed *p, spreg_packed_info *info) {
    clear_error();
    SPREG_CHECK_ARG(p && info, "null argument");
    *info = p->info;
    return SPREG_OK;
}

int spreg_packed_device_ptrs(const spreg_packed *p, const void **arena, const spreg_panel_desc **descs,
                             const float **scales) {
    clear_error();
    SPREG_CHECK_ARG(p, "null packed matrix");
    if (arena) *arena = p->arena;
    if (descs) *descs = p->descs;
    if (scales) *scales = p->scales;
    return SPREG_OK;
}

int spreg_packed_to_host(const spreg_packed *p, void *arena_host, int64_t arena_bytes, spreg_panel_desc *descs_host,
                         int64_t num_descs, float *scales_host, int64_t num_scales, spreg_stream_t stream) {
    clear_error();
    SPREG_CHECK_ARG(p, "null packed matrix");
    cudaStream_t s = (cudaStream_t)stream;
    if (arena_host) {
        SPREG_CHECK_ARG(arena_bytes >= p->info.arena_bytes, "arena buffer too small (%lld < %lld)",
                        (long long)arena_bytes, (long long)p->info.arena_bytes);
        if (p->info.arena_bytes)
            SPREG_CUDA(cudaMemcpyAsync(arena_host, p->arena, (size_t)p->info.arena_bytes, cudaMemcpyDeviceToHost, s));
    }
    if (descs_host) {
        SPREG_CHECK_ARG(num_descs >= p->info.num_units, "descriptor buffer too small");
        if (p->info.num_units)
            SPREG_CUDA(cudaMemcpyAsync(descs_host, p->descs, (size_t)p->info.num_units * sizeof(spreg_panel_desc),
                                       cudaMemcpyDeviceToHost, s));
    }
    if (scales_host && p->scales) {
        SPREG_CHECK_ARG(num_scales >= p->info.num_panels, "scales buffer too small");
        if (p->info.num_panels)
            SPREG_CUDA(cudaMemcpyAsync(scales_host, p->scales, (size_t)p->info.num_panels * sizeof(float),
                                       cudaMemcpyDeviceToHost, s));
    }
    SPREG_CUDA(cudaStreamSynchronize(s));
    return SPREG_OK;
}

// ---------------------------------------------------------------------- SOPTile
int spreg_tile_create(const spreg_mapping *m, int64_t rows, int64_t cols, int64_t num_panels, spreg_tile **out) {
    clear_error();
    SPREG_CHECK_ARG(out && m, "null argument");
    *out = nullptr;
    SPREG_CHECK_ARG(rows >= 0 && cols >= 0 && num_panels >= 0, "negative tile size");
    SPREG_CHECK_ARG(num_panels <= INT32_MAX, "too many panels");
    spreg_tile *t = new (std::nothrow) spreg_tile();
    if (!t) SPREG_FAIL(SPREG_ERR_NOMEM, "out of host memory");
    t->map = m;
    t->rows = rows;
    t->cols = cols;
    t->num_panels = num_panels;
    t->packed_flag.assign((size_t)num_panels, 0);
    t->codes.resize((size_t)num_panels);
    t->colidx.resize((size_t)num_panels);
    t->dense.resize((size_t)num_panels);
    t->panel_cols.assign((size_t)num_panels, 0);
    t->col_offset.assign((size_t)num_panels, 0);
    *out = t;
    return SPREG_OK;
}

int spreg_tile_pack_panel(spreg_tile *t, int64_t panel_id, int64_t col_offset, const int32_t *pat_codes,
                          const int32_t *col_indices, int64_t n, const float *dense_panel, int64_t panel_cols) {
    clear_error();
    SPREG_CHECK_ARG(t, "null tile");
    SPREG_CHECK_ARG(!t->packed, "tile already packed");
    // template:136-139
    SPREG_CHECK_ARG(panel_id >= 0 && panel_id < t->num_panels, "panel_id < num_panels failed (%lld, %lld)",
                    (long long)panel_id, (long long)t->num_panels);
    SPREG_CHECK_ARG(!t->packed_flag[(size_t)panel_id], "panel %lld already packed", (long long)panel_id);
    SPREG_CHECK_ARG(n >= 0 && panel_cols >= 0, "negative sizes");
    SPREG_CHECK_ARG(n == 0 || (pat_codes && col_indices), "null entry arrays");
    SPREG_CHECK_ARG(panel_cols == 0 || dense_panel, "null dense panel");
    SPREG_CHECK_ARG(col_offset >= 0 && panel_cols + col_offset <= INT32_MAX, "column indices must fit int32");
    const int mr = t->map->mr;
    for (int64_t i = 0; i < n; ++i) {
        const int32_t c = pat_codes[i];
        SPREG_CHECK_ARG(c >= 0 && c < (1 << mr) && t->map->code_to_id[c] != -1,
                        "pattern code %d is not a nanokernel of this module", c);
        SPREG_CHECK_ARG(col_indices[i] >= 0 && col_indices[i] < panel_cols,
                        "column index %d outside the dense panel (%lld columns)", col_indices[i], (long long)panel_cols);
    }
    const size_t p = (size_t)panel_id;
    t->codes[p].assign(pat_codes, pat_codes + n);
    t->colidx[p].assign(col_indices, col_indices + n);
    t->dense[p].assign(dense_panel, dense_panel + panel_cols * mr);
    t->panel_cols[p] = panel_cols;
    t->col_offset[p] = col_offset;
    t->packed_flag[p] = 1;
    return SPREG_OK;
}

int spreg_tile_pack(spreg_tile *t, int32_t value_dtype, spreg_stream_t stream) {
    clear_error();
    SPREG_CHECK_ARG(t, "null tile");
    SPREG_CHECK_ARG(!t->packed, "tile already packed");
    for (int64_t p = 0; p < t->num_panels; ++p)   // template:220
        SPREG_CHECK_ARG(t->packed_flag[(size_t)p], "panel %lld was not packed before pack_tile", (long long)p);
    std::vector<int32_t> codes, cols;
    std::vector<int64_t> eoff(1, 0), doff(1, 0);
    std::vector<float> dense;
    for (int64_t p = 0; p < t->num_panels; ++p) {
        codes.insert(codes.end(), t->codes[(size_t)p].begin(), t->codes[(size_t)p].end());
        cols.insert(cols.end(), t->colidx[(size_t)p].begin(), t->colidx[(size_t)p].end());
        eoff.push_back((int64_t)codes.size());
        dense.insert(dense.end(), t->dense[(size_t)p].begin(), t->dense[(size_t)p].end());
        doff.push_back((int64_t)dense.size());
    }
    doff.pop_back();
    spreg_packed *pk = nullptr;
    int st = pack_lists_impl(t->map, t->rows, t->cols, t->num_panels, codes, cols, eoff, dense, doff, t->panel_cols,
                             t->col_offset, value_dtype, &pk, (cudaStream_t)stream);
    if (st != SPREG_OK) return st;
    t->packed = pk;
    for (auto &v : t->codes) std::vector<int32_t>().swap(v);
    for (auto &v : t->colidx) std::vector<int32_t>().swap(v);
    for (auto &v : t->dense) std::vector<float>().swap(v);
    return SPREG_OK;
}

int64_t spreg_tile_padding(const spreg_tile *t) { return (t && t->packed) ? t->packed->info.padding : -1; }

const spreg_packed *spreg_tile_packed(const spreg_tile *t) { return t ? t->packed : nullptr; }

void spreg_tile_destroy(spreg_tile *t) {
    if (!t) return;
    packed_release(t->packed);
    delete t;
}

// ---------------------------------------------------------------------- executor
int spreg_execute(const spreg_packed *a, const spreg_exec_args *args, spreg_stream_t stream) {
    clear_error();
    return execute_impl(a, args, (cudaStream_t)stream);
}

int spreg_execute_explain(const spreg_packed *a, const spreg_exec_args *args, char *buf, int64_t len) {
    clear_error();
    return explain_impl(a, args, buf, len);
}

int spreg_load_balance_plan(const spreg_packed *a, const spreg_exec_args *args, int64_t *heavy_panels,
                            int32_t *split_tile, int32_t *heavy_ids, int64_t max_ids) {
    clear_error();
    return load_balance_plan_impl(a, args, heavy_panels, split_tile, heavy_ids, max_ids);
}

int spreg_execute_batched(const spreg_work_item *items, int32_t num_items, spreg_stream_t stream) {
    clear_error();
    return execute_batched_impl(items, num_items, (cudaStream_t)stream);
}

int spreg_device_status(int32_t *status, int32_t reset) {
    clear_error();
    return device_status_impl(status, reset);
}

int spreg_selftest_wait_timeout(uint32_t limit, int32_t *status_host, uint32_t *polls_host, spreg_stream_t stream) {
    clear_error();
    return selftest_wait_impl(limit, status_host, polls_host, (cudaStream_t)stream);
}

int spreg_execute_timed(const spreg_packed *a, const spreg_exec_args *args, int64_t num_runs, double *median_ns,
                        spreg_stream_t stream) {
    clear_error();
    return execute_timed_impl(a, args, num_runs, median_ns, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------- CSR baseline
int spreg_csr_spmm(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs,
                   const int32_t *col_inds, const float *values, const float *b, int64_t ldb, float *c, int64_t ldc,
                   int32_t n_tile, spreg_stream_t stream) {
    clear_error();
    return csr_spmm_impl(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, n_tile, (cudaStream_t)stream);
}

int spreg_csr_spmm_timed(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs,
                         const int32_t *col_inds, const float *values, const float *b, int64_t ldb, float *c,
                         int64_t ldc, int32_t n_tile, int64_t num_runs, double *median_ns, spreg_stream_t stream) {
    clear_error();
    return csr_spmm_timed_impl(rows, cols, n, nnz, row_ptrs, col_inds, values, b, ldb, c, ldc, n_tile, num_runs,
                               median_ns, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------- MatMulSpecialized
int spreg_matmul_create(int32_t m, int32_t k, int32_t n, const float *values, const int32_t *row_ptrs,
                        const int32_t *col_inds, const spreg_tile_config *cfg, const spreg_mapping *map,
                        spreg_matmul **out) {
    clear_error();
    SPREG_CHECK_ARG(out && map, "null argument");
    *out = nullptr;
    SPREG_CHECK_ARG(m >= 0 && k >= 0 && n >= 0, "negative sizes");
    SPREG_CHECK_ARG(m == 0 || row_ptrs, "null row_ptrs");
    const int64_t nnz = m > 0 ? row_ptrs[m] - row_ptrs[0] : 0;
    SPREG_CHECK_ARG(row_ptrs == nullptr || row_ptrs[0] == 0, "row_ptrs[0] must be 0");
    SPREG_CHECK_ARG(nnz >= 0, "row_ptrs must be non-decreasing");
    for (int32_t i = 0; i < m; ++i)
        SPREG_CHECK_ARG(row_ptrs[i + 1] >= row_ptrs[i], "row_ptrs must be non-decreasing (row %d)", i);
    SPREG_CHECK_ARG(nnz == 0 || (values && col_inds), "null values / col_inds");
    for (int64_t q = 0; q < nnz; ++q)
        SPREG_CHECK_ARG(col_inds[q] >= 0 && col_inds[q] < k, "column index %d out of range [0, %d)", col_inds[q], k);
    spreg_matmul *mm = new (std::nothrow) spreg_matmul();
    if (!mm) SPREG_FAIL(SPREG_ERR_NOMEM, "out of host memory");
    mm->m = m;
    mm->k = k;
    mm->n = n;
    if (cfg) mm->cfg = *cfg;
    if (mm->cfg.beta_10x == 0) mm->cfg.beta_10x = 10;
    cudaError_t e = cudaStreamCreateWithFlags(&mm->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete mm; SPREG_FAIL(SPREG_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
    int32_t *d_rp = nullptr, *d_ci = nullptr;
    float *d_v = nullptr;
    auto cleanup = [&]() {
        if (d_rp) cudaFree(d_rp);
        if (d_ci) cudaFree(d_ci);
        if (d_v) cudaFree(d_v);
    };
    e = cudaMalloc(&d_rp, (size_t)(m + 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_ci, (size_t)(nnz > 0 ? nnz : 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_v, (size_t)(nnz > 0 ? nnz : 1) * 4);
    if (e == cudaSuccess && m > 0) e = cudaMemcpy(d_rp, row_ptrs, (size_t)(m + 1) * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpy(d_ci, col_inds, (size_t)nnz * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpy(d_v, values, (size_t)nnz * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && m == 0) e = cudaMemset(d_rp, 0, 4);
    if (e != cudaSuccess) {
        cleanup();
        cudaStreamDestroy(mm->stream);
        delete mm;
        SPREG_FAIL(SPREG_ERR_CUDA, "CSR upload: %s", cudaGetErrorString(e));
    }
    spreg_csr csr{m, k, nnz, d_rp, d_ci, d_v};
    spreg_pack_opts o{mm->cfg.m_tile, mm->cfg.k_tile, 0, mm->cfg.value_dtype};
    int st = pack_csr_impl(map, &csr, &o, &mm->packed, mm->stream);
    cudaStreamSynchronize(mm->stream);
    cleanup();
    if (st != SPREG_OK) {
        cudaStreamDestroy(mm->stream);
        delete mm;
        return st;
    }
    // resolved configuration (get_config, SpMM_SOP.h:126-132)
    mm->cfg.m_tile = (int32_t)(mm->packed->geom.ppt * map->mr);
    mm->cfg.k_tile = (int32_t)mm->packed->geom.kt;
    if (mm->cfg.n_tile <= 0) mm->cfg.n_tile = n;
    *out = mm;
    return SPREG_OK;
}

int spreg_matmul_allocate_executor(spreg_matmul *mm, int32_t n) {
    clear_error();
    SPREG_CHECK_ARG(mm, "null matmul");
    SPREG_CHECK_ARG(n >= 0, "negative n");
    if (mm->alloc_n >= n && mm->dB) { mm->n = n; return SPREG_OK; }
    if (mm->dB) cudaFree(mm->dB);
    if (mm->dC) cudaFree(mm->dC);
    mm->dB = mm->dC = nullptr;
    SPREG_CUDA(cudaMalloc(&mm->dB, (size_t)std::max<int64_t>((int64_t)mm->k * n, 1) * 4));
    SPREG_CUDA(cudaMalloc(&mm->dC, (size_t)std::max<int64_t>((int64_t)mm->m * n, 1) * 4));
    mm->alloc_n = n;
    mm->n = n;
    return SPREG_OK;
}

// Job order of an outer schedule (tools/paper/configs.py:9-25, codes as spreg_tile_config documents):
// the K loop runs inside every job (K tiles accumulate in registers), so what a schedule decides on
// the GPU is whether the N loop (column strips) is outside the M loop (row panels).
static int32_t job_order_of_schedule(int32_t sched) {
    static const char *const names[] = {"KNM", "NKM", "MNK", "NMK", "KMN", "MKN", "KM", "MK",
                                        "KN",  "NK",  "MN",  "NM",  "K",   "N",   "M"};
    if (sched < 0 || sched >= (int32_t)(sizeof names / sizeof names[0])) return 0;
    const char *n = names[sched];
    const char *pn = std::strchr(n, 'N'), *pm = std::strchr(n, 'M');
    return (pn && (!pm || pn < pm)) ? 1 : 0;
}

static int matmul_exec(spreg_matmul *mm, float *c, const float *b, cudaStream_t s) {
    spreg_exec_args a = {};
    a.job_order = job_order_of_schedule(mm->cfg.outer_schedule);
    a.load_balance = mm->cfg.load_balance;
    a.b = b;
    a.ldb = mm->n;
    a.c = c;
    a.ldc = mm->n;
    a.n = mm->n;
    a.b_dtype = mm->cfg.value_dtype;
    a.c_dtype = SPREG_F32;
    a.load_c = 0;
    a.nr = mm->cfg.nr;
    return execute_impl(mm->packed, &a, s);
}

static int matmul_enqueue(spreg_matmul *mm, float *c_host, const float *b_host) {
    SPREG_CHECK_ARG(mm, "null matmul");
    SPREG_CHECK_ARG(mm->cfg.value_dtype == SPREG_F32, "host operator() takes FP32 buffers; use run_device for 16-bit B");
    if (!mm->dB || mm->alloc_n < mm->n) {
        int st = spreg_matmul_allocate_executor(mm, mm->n);
        if (st) return st;
    }
    SPREG_CHECK_ARG(c_host && (b_host || mm->k == 0 || mm->n == 0), "null host buffers");
    const size_t bb = (size_t)mm->k * mm->n * 4, cb = (size_t)mm->m * mm->n * 4;
    if (bb) SPREG_CUDA(cudaMemcpyAsync(mm->dB, b_host, bb, cudaMemcpyHostToDevice, mm->stream));
    // direct output: the kernel's stores of C cross to host memory themselves, beside the copy
    // engines that carry the other calls' C
    const bool direct = mm->direct_output && cb && host_mapped(c_host);
    int st = matmul_exec(mm, direct ? c_host : mm->dC, mm->dB, mm->stream);
    if (st) return st;
    if (cb && !direct) SPREG_CUDA(cudaMemcpyAsync(c_host, mm->dC, cb, cudaMemcpyDeviceToHost, mm->stream));
    return SPREG_OK;
}

int spreg_matmul_set_direct_output(spreg_matmul *mm, int32_t direct) {
    clear_error();
    SPREG_CHECK_ARG(mm, "null matmul");
    mm->direct_output = direct ? 1 : 0;
    return SPREG_OK;
}

int spreg_matmul_run_async(spreg_matmul *mm, float *c_host, const float *b_host) {
    clear_error();
    return matmul_enqueue(mm, c_host, b_host);
}

int spreg_matmul_sync(spreg_matmul *mm) {
    clear_error();
    SPREG_CHECK_ARG(mm, "null matmul");
    SPREG_CUDA(cudaStreamSynchronize(mm->stream));
    return SPREG_OK;
}

int spreg_matmul_run(spreg_matmul *mm, float *c_host, const float *b_host) {
    clear_error();
    int st = matmul_enqueue(mm, c_host, b_host);
    if (st) return st;
    SPREG_CUDA(cudaStreamSynchronize(mm->stream));
    return SPREG_OK;
}

int spreg_matmul_run_device(spreg_matmul *mm, float *c, const float *b, spreg_stream_t stream) {
    clear_error();
    SPREG_CHECK_ARG(mm, "null matmul");
    return matmul_exec(mm, c, b, (cudaStream_t)stream);
}

int spreg_matmul_get_config(const spreg_matmul *mm, spreg_tile_config *cfg) {
    clear_error();
    SPREG_CHECK_ARG(mm && cfg, "null argument");
    *cfg = mm->cfg;
    return SPREG_OK;
}

int64_t spreg_matmul_required_storage(const spreg_matmul *mm) {
    return (mm && mm->packed) ? mm->packed->info.required_storage : -1;
}

const spreg_packed *spreg_matmul_packed(const spreg_matmul *mm) { return mm ? mm->packed : nullptr; }

void spreg_matmul_destroy(spreg_matmul *mm) {
    if (!mm) return;
    if (mm->stream) cudaStreamSynchronize(mm->stream);
    packed_release(mm->packed);
    if (mm->dB) cudaFree(mm->dB);
    if (mm->dC) cudaFree(mm->dC);
    if (mm->stream) cudaStreamDestroy(mm->stream);
    delete mm;
}

}  // extern "C"
