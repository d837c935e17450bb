/*
 * spreg.h -- C ABI of the GB300 sparse-register-tiling SpMM library (libspreg.so).
 *
 * The library packs a pruned sparse weight A once ("inspector") and multiplies the packed
 * form against dense B on an sm_103a GPU ("executor").  Every entry point takes plain
 * pointers and sizes, returns an int status (SPREG_OK == 0) and never exits the process;
 * the message of the last failure on the calling thread is spreg_last_error().
 *
 * Pointer convention: arrays named *_host are host memory; every other array pointer is
 * device memory of the current CUDA device.  Every device entry point takes an explicit
 * stream (a cudaStream_t; NULL is the legacy default stream).
 *
 * Reference interfaces this ABI replaces (paths inside the reference project):
 *   - sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:84-98, 101-262, 351-392, 396-409
 *     (sort_and_encode_patterns, SOPTile.pack_panel / pack_tile / padding, execute_tile)
 *   - sbench/SOP/sop_driver.py:38-129 (make_sop_module, SOPModule.make_sop_tile)
 *   - cpp_testbed/src/spmm/nano/SpMM_SOP.h:107-178 (sop::MatMulSpecialized constructor,
 *     get_config, allocate_executor, operator()(C, B), require_storage)
 *   - cpp_testbed/demo/count_nkerns.cpp:52-128 (tiled packer: M_c x K_c tiles, load_c)
 *   - sbench/SOP/_C/pytorch_csr_wrapper.cpp:70-191, 314-353 (the csr module's executor: the CSR
 *     baseline that sbench/SOP/sop_bench.py:197 times beside the register-tiled executor)
 *
 * Device status word: kernels never trap.  A bounded wait that gives up, or an index a kernel's
 * own bounds check refuses, records a nonzero code in a per-device word instead (read and clear it
 * with spreg_device_status):
 *   2, 5-9   executor waits (batched and B-tile kernels);   20  CSR column index out of range;
 *   21-25    tensor-core kernel waits;                         30  spreg_selftest_wait_timeout.
 */
#ifndef SPREG_H
#define SPREG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t; declared here so callers need no CUDA header. */
typedef struct CUstream_st *spreg_stream_t;

/* ---------------------------------------------------------------- status codes */
enum {
    SPREG_OK = 0,
    SPREG_ERR_INVALID_ARG = 1, /* bad argument (reference: TORCH_CHECK failure) */
    SPREG_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    SPREG_ERR_UNSUPPORTED = 3, /* valid request outside what this build supports */
    SPREG_ERR_STATE = 4,       /* call out of order (e.g. execute before pack_tile) */
    SPREG_ERR_CHECK = 5,       /* a device-side check failed (packer invariant, bad code) */
    SPREG_ERR_NOMEM = 6        /* device allocation failed */
};

typedef enum {
    SPREG_F32 = 0,  /* float */
    SPREG_BF16 = 1, /* bfloat16, FP32 accumulation */
    SPREG_F16 = 2   /* IEEE half with a power-of-two scale per row panel, FP32 accumulation */
} spreg_dtype;

/* Encoded id of the all-zero pattern; sorts after every nanokernel id (template:77). */
#define SPREG_ZERO_PATTERN_ID 0xFFFF
/* Largest supported panel height M_r (patterns are M_r-bit masks). */
#define SPREG_MAX_MR 8

/* Message of the last failed call on this thread ("" if none). */
const char *spreg_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int spreg_version(void);

/* ------------------------------------------------- nanokernel set + pattern mapping
 * A mapping sends every M_r-bit column pattern p in [0, 2^M_r) to a list of nanokernel
 * patterns; the column is emitted once per listed pattern (sop_driver.py:50-65).  Lists
 * live in map_codes[map_offsets[p] .. map_offsets[p+1]).  A listed 0 drops the column.
 * The nanokernel set is `nanokernels` (the module's `patterns`, sop_driver.py:88-106) or,
 * if NULL, every distinct nonzero pattern that the mapping lists.  Nanokernel ids are the
 * set sorted by (popcount, value); that order is this library's definition of
 * MicroKernel::encode_nkern_pattern, whose source is absent from the reference.
 */
typedef struct spreg_mapping spreg_mapping;

int spreg_mapping_create(int32_t mr, const int32_t *map_offsets_host, const int32_t *map_codes_host,
                         const int32_t *nanokernels_host, int32_t num_nanokernels, spreg_mapping **out);
void spreg_mapping_destroy(spreg_mapping *m);
int32_t spreg_mapping_mr(const spreg_mapping *m);
/* MicroKernel::num_nkern_patterns() (template:44). */
int32_t spreg_mapping_num_nkern(const spreg_mapping *m);
/* out_host[id] = nanokernel pattern of id (MicroKernel::decode_nkern_pattern). */
int spreg_mapping_nkern_patterns(const spreg_mapping *m, int32_t *out_host);
/* MicroKernel::encode_nkern_pattern: id, SPREG_ZERO_PATTERN_ID for 0, -1 if not in the set. */
int32_t spreg_mapping_encode(const spreg_mapping *m, int32_t pattern);

/* sort_and_encode_patterns (template:84-98): encoded[i] = encode(pat_codes[order[i]]) with
 * `order` the stable sort of the encoded ids, zero pattern last.  Device arrays of n. */
int spreg_sort_and_encode_patterns(const spreg_mapping *m, const int32_t *pat_codes, int64_t n,
                                   int32_t *encoded, int32_t *order, spreg_stream_t stream);

/* ------------------------------------------------------------------ packed matrix
 * A packed matrix is the reference's SOPTile arena (template:219-261): for every packed
 * unit (one M_r-row panel, or one panel of one M_c x K_c tile) in order
 *   [values | pad to 64 B | col_indices (int32) | pad to 64 B | nkern_counts (int32) | pad to 64 B]
 * with values in ascending-row order per entry and entries stably sorted by nanokernel id.
 * Units are ordered row tile, then K tile, then panel (count_nkerns.cpp:78-125).
 */
typedef struct spreg_packed spreg_packed;

typedef struct {
    int64_t values_off; /* byte offset of the unit's values in the arena */
    int64_t cols_off;   /* byte offset of the unit's col_indices */
    int64_t counts_off; /* byte offset of the unit's nkern_counts */
    int32_t num_values; /* MicroKernelPackedData::num_nnz (includes padding zeros) */
    int32_t num_cols;   /* MicroKernelPackedData::num_col_indices */
} spreg_panel_desc;

typedef struct {
    int64_t rows, cols;        /* M, K of A */
    int64_t num_panels;        /* ceil(M / M_r) row panels */
    int64_t num_units;         /* packed units = descriptors */
    int32_t mr, num_nkern;
    int32_t m_tile, k_tile;    /* M_c, K_c (rows / columns per tile) */
    int32_t num_k_tiles;       /* K tiles per row tile */
    int32_t value_dtype;       /* spreg_dtype of the stored values */
    int64_t col_offset;        /* added to every stored column index */
    int64_t nnz;               /* nonzeros of A */
    int64_t num_values;        /* sum of num_values (nnz + padding) */
    int64_t num_col_indices;   /* sum of num_cols */
    int64_t padding;           /* emitted zero values (SOPTile::padding) */
    int64_t arena_bytes;       /* bytes of the arena */
    int64_t required_storage;  /* reference bound sum(values + cols + counts + 3*64) (template:222-229) */
    int64_t algorithmic_bytes; /* values + col indices + counts + descriptors + scales */
    int64_t empty_units;       /* units of tiles with no nonzero (EMPTY_TILE, count_nkerns.cpp:114-117) */
} spreg_packed_info;

typedef struct {
    int64_t rows, cols, nnz;
    const int32_t *row_ptrs; /* rows + 1 */
    const int32_t *col_inds; /* nnz, any order within a row, no duplicates */
    const float *values;     /* nnz; explicit zeros are treated as zeros */
} spreg_csr;

typedef struct {
    int32_t m_tile;      /* M_c, multiple of M_r; 0 = one row tile */
    int32_t k_tile;      /* K_c; 0 = one K tile */
    int64_t col_offset;  /* added to stored column indices (SOPTile.pack_panel col_offset) */
    int32_t value_dtype; /* spreg_dtype of stored values */
} spreg_pack_opts;

/* Pack a CSR matrix (device arrays) -- the MicroKernelPacker / MatMulSpecialized inspector. */
int spreg_pack_csr(const spreg_mapping *m, const spreg_csr *a, const spreg_pack_opts *opts,
                   spreg_packed **out, spreg_stream_t stream);
/* Pack a dense row-major M x K matrix (device, leading dimension lda); nonzeros define patterns. */
int spreg_pack_dense(const spreg_mapping *m, const float *a, int64_t rows, int64_t cols, int64_t lda,
                     const spreg_pack_opts *opts, spreg_packed **out, spreg_stream_t stream);
void spreg_packed_destroy(spreg_packed *p);
int spreg_packed_get_info(const spreg_packed *p, spreg_packed_info *info);
/* Device pointers of the arena, the descriptors and (F16 only, else NULL) per-panel scales. */
int spreg_packed_device_ptrs(const spreg_packed *p, const void **arena, const spreg_panel_desc **descs,
                             const float **scales);
/* Copy arena, descriptors and scales to host buffers (any may be NULL); synchronises `stream`. */
int spreg_packed_to_host(const spreg_packed *p, void *arena_host, int64_t arena_bytes,
                         spreg_panel_desc *descs_host, int64_t num_descs, float *scales_host,
                         int64_t num_scales, spreg_stream_t stream);

/* Geometry an arena was packed with (spreg_pack_opts plus A's shape). */
typedef struct {
    int64_t rows, cols;      /* A is rows x cols */
    int32_t m_tile, k_tile;  /* M_c, K_c (0: one tile) */
    int64_t col_offset;
    int32_t value_dtype;
    int32_t reserved;        /* 0 */
} spreg_arena_geom;

/* Rebuild a packed matrix from host copies of an earlier packing's arena, descriptors and F16
 * scales (spreg_packed_to_host), e.g. read back from a file.  The arena keeps the byte layout of
 * SOPTile::pack_tile (sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:219-261); the executor's
 * layout is rebuilt from it on the device.  Every unit is checked (descriptors inside the arena
 * and equal to the layout of their counts, counts adding up to the unit's columns and values,
 * columns inside the unit's K tile); a failed check is SPREG_ERR_CHECK.  Synchronises `stream`. */
int spreg_pack_from_arena(const spreg_mapping *m, const spreg_arena_geom *geom, const void *arena_host,
                          int64_t arena_bytes, const spreg_panel_desc *descs_host, int64_t num_units,
                          const float *scales_host, int64_t num_scales, spreg_packed **out, spreg_stream_t stream);

/* ---------------------------------------------------------- SOPTile (Python path)
 * Mirrors SOPTile(rows, cols, num_panels).pack_panel(...) / pack_tile() / padding()
 * (template:101-262).  pack_panel takes host arrays: n (code, column) entries in caller
 * order and the panel's dense values, dense_panel_host[c * M_r + r] for c < panel_cols.
 * pack_panel validates and stages; pack_tile runs the GPU packer over all panels.
 */
typedef struct spreg_tile spreg_tile;

int spreg_tile_create(const spreg_mapping *m, int64_t rows, int64_t cols, int64_t num_panels,
                      spreg_tile **out);
int spreg_tile_pack_panel(spreg_tile *t, int64_t panel_id, int64_t col_offset, const int32_t *pat_codes_host,
                          const int32_t *col_indices_host, int64_t n, const float *dense_panel_host,
                          int64_t panel_cols);
int spreg_tile_pack(spreg_tile *t, int32_t value_dtype, spreg_stream_t stream);
/* Padding zeros of the packed tile (valid after spreg_tile_pack; -1 before). */
int64_t spreg_tile_padding(const spreg_tile *t);
/* The packed matrix of a packed tile (owned by the tile), NULL before spreg_tile_pack. */
const spreg_packed *spreg_tile_packed(const spreg_tile *t);
void spreg_tile_destroy(spreg_tile *t);

/* ------------------------------------------------------------------------ executor */
enum { SPREG_EPILOGUE_NONE = 0, SPREG_EPILOGUE_RELU = 1 };

typedef struct {
    const void *b;       /* K x ldb row-major, element type b_dtype (same family as the values) */
    int64_t ldb;
    void *c;             /* M x ldc row-major, element type c_dtype (F32 or BF16) */
    int64_t ldc;
    int64_t n;           /* columns of B and C to compute (N_c) */
    int32_t b_dtype, c_dtype;
    int32_t load_c;      /* 1: C += A.B (template:290-297 load_c) ; 0: C = A.B */
    int32_t epilogue;    /* SPREG_EPILOGUE_* applied to the stored result */
    int32_t nr;          /* columns per warp strip: 32, 64, 128, 256 or 512; 0 = automatic.  256 and
                            512 are wide strips where a kernel has them, else 128: the B-tile kernel
                            with 16-bit B (256); the gather kernel with FP32 values, B and C, 16-byte
                            aligned B and C with row strides in whole 16-byte units (256; 512 at
                            M_r <= 4), its lanes holding interleaved 16-byte quarters of the strip,
                            and with 16-bit B at M_r <= 4 (256; 512: 8 columns a lane in each
                            256-column half) */
    int32_t warps_per_cta; /* CTA tiling, 1..8; 0 = automatic: warps per CTA of the batched and
                              register-stream kernels (8 and 4 by default), consumer warps (row panels
                              per job) of the B-tile kernel (15 by default) */
    int32_t b_staging;   /* 0 automatic, 1 stage B strips in shared memory (bulk copies), 2 read B via L1/L2 */
    int32_t meta_staging; /* 0 automatic, 1 stage each panel's execution block in shared memory, 2 stream
                             the packed arena through registers */
    int32_t job_order;   /* order in which the (row panel, column strip) jobs are handed out: 0 = row
                            panels outer (a panel's strips one after another, its metadata reused), 1 =
                            column strips outer (a strip of B reused across panels).  Results do not
                            depend on it (each element's FMA order is fixed). */
    int32_t panel_rounds; /* 0 or 1: one round; R > 1 (<= 64): the B-tile kernel keeps a job's strip of B
                             for every K tile resident in shared memory while R rounds of its consumer
                             warps' panels run against it (B read from L2 once per R x warps panels).
                             Needs b_staging 0 or 1 and a strip (K x 32 * nr/32 columns) that fits
                             shared memory; results do not depend on it. */
    int32_t load_balance; /* 0: off.  1: split the heaviest row panels' K tiles between two concurrent jobs
                             (the reference's load-balanced kernel choice, KD_IntelLoadBalanced in
                             cpp_testbed/src/spmm/nano/runtime_yaml_config.register:84-99).  When the
                             launch leaves SMs idle (fewer jobs of W panels x strips than SMs), the
                             heaviest whole groups of W panels (work estimate above half the heaviest
                             panel's) are split at K tile T / 2 until the idle SMs are used, unless
                             some groups stay unsplit and the first of them is within a fifth of the
                             heaviest panel, or the heaviest panel's work is below twice the median
                             panel's: K tiles
                             [0, T/2) accumulate into C (from C with load_c) in one job, tiles [T/2, T)
                             from zero in another, which adds into C once the first has stored that
                             (panel, strip): C = C + hi, one FP32 add per element, the epilogue after
                             it, all in one launch.  Needs a K-tiled pack (T >= 2) of FP32 or BF16 values, FP32 C
                             and the B-tile kernel (b_staging 0 or 1); other packs run unsplit.
                             The two halves meet through flags from a per-device pool that a call
                             reuses only after at least 64 others (as the executors' work counters
                             after 4096 launches), so fewer load-balanced calls than that may be in
                             flight on the GPU at once.  spreg_load_balance_plan reports the split. */
    int32_t reserved;     /* 0 */
} spreg_exec_args;

/* One SpMM: C (+)= A . B over the first n columns -- sop_multiple_panel_executor (template:265-305). */
int spreg_execute(const spreg_packed *a, const spreg_exec_args *args, spreg_stream_t stream);

/* The plan spreg_execute(a, args) would make, as one line of text into buf (len bytes): the kernel,
 * M_r, strip width, main / tail columns, K tiles, warps, panel rounds and load-balanced split.
 * Checks the arguments as spreg_execute does; no launch. */
int spreg_execute_explain(const spreg_packed *a, const spreg_exec_args *args, char *buf, int64_t len);

/* The load-balanced split spreg_execute(a, args) would make (as with args->load_balance = 1), the
 * call running alone: *heavy_panels panels are split at K tile *split_tile (0 and 0: no split);
 * heavy_ids (may be NULL, else room for max_ids) receives their row-panel indices.  No launch. */
int spreg_load_balance_plan(const spreg_packed *a, const spreg_exec_args *args, int64_t *heavy_panels,
                            int32_t *split_tile, int32_t *heavy_ids, int64_t max_ids);

/* Many SpMMs of uneven shape in ONE launch, from a (matrix, panel, column-strip) work list. */
typedef struct {
    const spreg_packed *a;
    spreg_exec_args args;
} spreg_work_item;

int spreg_execute_batched(const spreg_work_item *items_host, int32_t num_items, spreg_stream_t stream);

/* Executor for callers that cannot allocate device memory while they run it (a serving loop whose
 * memory belongs to another allocator, or a path that must not add the synchronisation a first
 * cudaMalloc can cause).  Same work list and results as spreg_execute_batched, but it calls no
 * cudaMalloc / cudaFree: its scratch (a status word and one work counter per launch) is a static
 * device array of SPREG_NOALLOC_MAX_LAUNCHES + 1 ints that every GPU loading the library keeps
 * until exit.  A list that needs more than SPREG_NOALLOC_MAX_LAUNCHES launches (one launch per
 * group of up to 224 SpMMs of one M_r / strip width / dtype combination) is rejected.  The first
 * call on each device looks up the array's device address; make it before any stream capture.
 * Calls share the array and clear its counters at their start, so calls that overlap on the GPU
 * race.  Its status word (a bounded wait that gave up) is read and cleared by spreg_device_status,
 * like the regular executors' word, and keeps its value until then.  It runs only the batched
 * execution-layout kernel (no meta_staging = 2, no oversized blocks): where spreg_execute_batched's
 * automatic B staging picks the shared-memory B-tile kernel (K-tiled packs), this entry point gives
 * the same results from the batched kernel, more slowly.  Strip widths (nr, the wide strips of
 * 256 and 512 columns included) are chosen as spreg_execute chooses them for the batched kernel.
 * It has no counterpart in the reference. */
#define SPREG_NOALLOC_MAX_LAUNCHES 64
int spreg_execute_batched_noalloc(const spreg_work_item *items_host, int32_t num_items, spreg_stream_t stream);

/* Dense row panels on the tensor cores: C[row_index[i], 0:n] (+)= A_rows[i, 0:k] . B[0:k, 0:n] for
 * i < rows, with tcgen05 BF16 MMAs accumulating in FP32 tensor memory (all pointers on the device).
 * A_rows is rows x k BF16 (16-byte aligned, lda a multiple of 8), B is k x n BF16 (row stride ldb), C
 * is F32 or BF16 (row stride ldc); load_c adds C, epilogue 1 applies ReLU.  For the panels of a
 * pruned matrix dense enough that a dense product beats the register-tiled executors (the
 * reference's executor runs every panel register-tiled, spmm/nano/SpMM_SOP.h:174-178).  Results
 * are not bit-identical to the register-tiled order: the accumulation order is the tensor core's. */
int spreg_dense_rows_bf16(const void *a_rows, int64_t rows, int64_t k, int64_t lda, const int32_t *row_index,
                          const void *b, int64_t ldb, void *c, int64_t ldc, int64_t n, int32_t c_dtype,
                          int32_t load_c, int32_t epilogue, spreg_stream_t stream);

/* One product of spreg_dense_rows_bf16, for the batched call. */
typedef struct {
    const void *a_rows;
    int64_t rows, k, lda;
    const int32_t *row_index;
    const void *b;
    int64_t ldb;
    void *c;
    int64_t ldc, n;
    int32_t c_dtype, load_c, epilogue;
    int32_t tile_n;          /* output tile width: 0 = automatic, 128 or 256 (a launch takes the first
                                nonzero hint of its items) */
} spreg_dense_rows_item;

/* Many dense-rows products (any shapes) in as few launches as possible: the output tiles of up to
 * 192 products share one launch.  Same arguments and results as spreg_dense_rows_bf16 per item. */
int spreg_dense_rows_bf16_batched(const spreg_dense_rows_item *items, int32_t num_items, spreg_stream_t stream);

/* FP32-accurate dense rows on the tensor cores.  The FP32 executor's accuracy at tensor-core rate: A
 * (per row) and B (per column) are scaled by powers of two and split into FP16 halves, x = hi + lo,
 * and each product runs as hi.hi + hi.lo + lo.hi FP16 MMAs with FP32 accumulation.  The terms left
 * out are below 2^-22 of each product.  The tensor core's FP32 accumulation truncates, so its error
 * grows with the 16-deep K steps of one accumulator: products with k > 1024 run as passes over K
 * chunks of 1024, each adding into C, which keeps the result within the FP32 executor's tolerance
 * (rel err <= 1e-5) at any K.  Not bit-identical to the register-tiled order.
 * Values whose magnitude is more than 2^17 below their row's (A) or column's (B) largest keep an
 * absolute error below 2^-25 of the scaled unit; scales are limited to 2^-126 .. 2^126.
 *
 * spreg_dense_rows_f32_split prepares the A side once (a pruned weight's dense panels): a_rows is
 * rows x k FP32 (row stride lda); a_split receives 2 * rows rows of ld_split FP16 (16-byte aligned,
 * ld_split >= k a multiple of 8): rows [0, rows) the high halves, [rows, 2 rows) the low halves;
 * row_scale[i] receives 2^-s of row i's scale. */
int spreg_dense_rows_f32_split(const float *a_rows, int64_t rows, int64_t k, int64_t lda, void *a_split,
                               int64_t ld_split, float *row_scale, spreg_stream_t stream);

/* One FP32-accurate product: C[row_index[i], 0:n] (+)= A_rows[i, 0:k] . B[0:k, 0:n] with A_rows given
 * as its split pair; B is FP32 k x n (row stride ldb), C FP32 (row stride ldc). */
typedef struct {
    const void *a_split;     /* spreg_dense_rows_f32_split output: 2 * rows x ld_split FP16 */
    int64_t rows, k, ld_split;
    const float *row_scale;  /* rows */
    const int32_t *row_index;
    const float *b;
    int64_t ldb;
    float *c;
    int64_t ldc, n;
    int32_t load_c, epilogue;
    int32_t tile_n;          /* output tile width: 0 = automatic, 128 or 256 */
    int32_t reserved;        /* 0 */
} spreg_dense_rows_f32_item;

/* One product / many products in as few launches as possible (B of each product is split into its
 * FP16 pair by one preparation launch, then the output tiles of up to 192 products share one
 * tensor-core launch).  Products with the same A, row index, load_c and epilogue coalesce into one
 * product over their side-by-side B. */
int spreg_dense_rows_f32(const spreg_dense_rows_f32_item *item, spreg_stream_t stream);
int spreg_dense_rows_f32_batched(const spreg_dense_rows_f32_item *items, int32_t num_items, spreg_stream_t stream);

/* A reusable plan of spreg_dense_rows_f32_batched / spreg_dense_rows_bf16_batched for a fixed item
 * list (the same pointers every run): its scratch, tensor maps and device tables are made once
 * (synchronising `stream`), so a run is its kernel launches (B preparation, tensor-core launches)
 * and no host-side work, and can be captured in a CUDA graph.  The plan belongs to the device
 * current at creation; runs of one plan must not overlap on the GPU (they share its scratch). */
typedef struct spreg_dense_rows_plan spreg_dense_rows_plan;
int spreg_dense_rows_f32_plan_create(const spreg_dense_rows_f32_item *items, int32_t num_items,
                                     spreg_dense_rows_plan **out, spreg_stream_t stream);
int spreg_dense_rows_bf16_plan_create(const spreg_dense_rows_item *items, int32_t num_items,
                                      spreg_dense_rows_plan **out, spreg_stream_t stream);
int spreg_dense_rows_plan_run(const spreg_dense_rows_plan *plan, spreg_stream_t stream);
void spreg_dense_rows_plan_destroy(spreg_dense_rows_plan *plan);

/* Status word of the current device: nonzero once a kernel gave up a bounded wait (its results
 * are then incomplete) -- the regular kernels' word, or, when that is 0, the word of
 * spreg_execute_batched_noalloc.  Synchronous; reset != 0 clears both. */
int spreg_device_status(int32_t *status_host, int32_t reset);

/* Self-test of the bounded waits every kernel uses: one CTA waits on an mbarrier that nothing
 * arrives on, polling `limit` times (1 .. 2^22).  The wait gives up, the kernel records 30 in the
 * device status word and returns; *status_host receives the status word and *polls_host the polls
 * made.  Synchronous.  The context stays usable (clear the word with spreg_device_status(.., 1)). */
int spreg_selftest_wait_timeout(uint32_t limit, int32_t *status_host, uint32_t *polls_host, spreg_stream_t stream);

/* execute_tile (template:351-392): C = A.B over n_c columns, timed: warm-up num_runs runs,
 * then 150 x num_runs timed runs; *median_ns = median per-run time in nanoseconds. */
int spreg_execute_timed(const spreg_packed *a, const spreg_exec_args *args, int64_t num_runs,
                        double *median_ns, spreg_stream_t stream);

/* ------------------------------------------- CSR baseline (the reference's csr module) */
/* C = A.B for a CSR A (rows x cols, nnz entries, device arrays) and B (cols x n, ldb), FP32,
 * row x N-tile FMAs in CSR order from zero: pytorch_csr_wrapper.cpp:70-191 (kernel) and :314-353
 * (csr.executor, as sbench/SOP/sop_bench.py:197 calls it).  n_tile is the reference's tile of
 * 16 / 32 / 64 / 128 floats; it sets the strip width, never the result.  Row pointers are clamped
 * to [0, nnz]; a column index outside [0, cols) contributes nothing and sets the device status
 * word (20). */
int spreg_csr_spmm(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs,
                   const int32_t *col_inds, const float *values, const float *b, int64_t ldb, float *c, int64_t ldc,
                   int32_t n_tile, spreg_stream_t stream);
/* profile() of pytorch_csr_wrapper.cpp:200-232: num_runs warm-up runs, then 150 x num_runs timed
 * runs; *median_ns = the median per run (ns).  C holds one product afterwards. */
int spreg_csr_spmm_timed(int64_t rows, int64_t cols, int64_t n, int64_t nnz, const int32_t *row_ptrs,
                         const int32_t *col_inds, const float *values, const float *b, int64_t ldb, float *c,
                         int64_t ldc, int32_t n_tile, int64_t num_runs, double *median_ns, spreg_stream_t stream);

/* ------------------------------------------- MatMulSpecialized (C++ path, host buffers) */
typedef struct {
    int32_t m_tile, k_tile, n_tile; /* M_c, K_c, N_c (SOPConfig m_tile/k_tile/n_tile) */
    int32_t nr;                     /* columns per warp strip, 0 = automatic */
    int32_t outer_schedule;         /* KNM=0, NKM=1, MNK=2, NMK=3, KMN=4, MKN=5, KM=6, MK=7, KN=8, NK=9, MN=10,
                                       NM=11, K=12, N=13, M=14 (tools/paper/configs.py:9-25): K runs inside
                                       every GPU job, so a schedule with N outside M hands out column
                                       strips outer (job_order 1), the others row panels outer */
    int32_t value_dtype;            /* spreg_dtype of stored values */
    int32_t sparse_a, tiling_strategy, beta_10x; /* accepted and reported; no GPU effect */
    int32_t load_balance;           /* the load-balanced kernel (runtime_yaml_config.register:84-99): as
                                       spreg_exec_args.load_balance */
} spreg_tile_config;

typedef struct spreg_matmul spreg_matmul;

/* sop::MatMulSpecialized(m, k, n, values, row_ptrs, col_inds, TileConfig, ...) with HOST CSR. */
int spreg_matmul_create(int32_t m, int32_t k, int32_t n, const float *values_host, const int32_t *row_ptrs_host,
                        const int32_t *col_inds_host, const spreg_tile_config *cfg, const spreg_mapping *map,
                        spreg_matmul **out);
/* allocate_executor(n): device staging for B (k x n) and C (m x n). */
int spreg_matmul_allocate_executor(spreg_matmul *mm, int32_t n);
/* operator()(C, B) with HOST buffers: copy B in, C = A.B, copy C out (synchronous). */
int spreg_matmul_run(spreg_matmul *mm, float *c_host, const float *b_host);
/* operator()(C, B) with HOST buffers, enqueued on the matmul's own stream without waiting: the copy in,
 * the product and the copy out run in order there, overlapping other matmuls' copies and products.
 * b_host and c_host must stay valid until spreg_matmul_sync; pinned buffers make the copies
 * asynchronous (pageable ones are staged synchronously by the driver).  Same result as
 * spreg_matmul_run. */
int spreg_matmul_run_async(spreg_matmul *mm, float *c_host, const float *b_host);
/* Wait for every call enqueued on the matmul's stream; then c_host of those calls holds C. */
int spreg_matmul_sync(spreg_matmul *mm);
/* direct != 0 (the default): host-buffer calls whose c_host is page-locked host memory the device
 * maps at the same address (cudaHostAlloc, torch pin_memory) have the kernel store C straight into
 * it: no device C and no copy out.  Any other c_host takes the copy path (device C, then a copy).
 * Results are identical either way; direct = 0 keeps the copy path for every call. */
int spreg_matmul_set_direct_output(spreg_matmul *mm, int32_t direct);
/* Same on device buffers (ldb = ldc = n), asynchronous on `stream`. */
int spreg_matmul_run_device(spreg_matmul *mm, float *c, const float *b, spreg_stream_t stream);
int spreg_matmul_get_config(const spreg_matmul *mm, spreg_tile_config *cfg);
/* require_storage: the packed bound (template:222-229 summed over tiles). */
int64_t spreg_matmul_required_storage(const spreg_matmul *mm);
const spreg_packed *spreg_matmul_packed(const spreg_matmul *mm);
void spreg_matmul_destroy(spreg_matmul *mm);

#ifdef __cplusplus
}
#endif

#endif /* SPREG_H */
