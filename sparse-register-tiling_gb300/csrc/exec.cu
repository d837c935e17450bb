// exec.cu -- host side of the executor: argument checks, strip widths, work lists, launches.
//
// Every SpMM call becomes one or two "problems" of the batched persistent kernel
// (exec_batch_kernel): whole column strips of 32 * NV columns, plus an NV = 1 problem for the
// columns past the last whole strip.  spreg_execute_batched groups the problems of many SpMMs by
// kernel configuration (M_r, NV, data types) and runs each group in one launch.  Packs whose
// execution blocks do not fit the per-warp buffers, or calls that ask for it (meta_staging = 2),
// run the register-stream kernel (exec_kernel) instead.  Calls with b_staging = 1 run the
// shared-memory B-tile kernel (exec_tile_kernel), grouped the same way.
#include "exec_tile.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace spreg {

namespace {

int combo_of(int vt, int bt, int ct) {
    if (vt == SPREG_F32 && bt == SPREG_F32 && ct == SPREG_F32) return COMBO_F32;
    if (vt == SPREG_BF16 && bt == SPREG_BF16 && ct == SPREG_F32) return COMBO_BF16_F32OUT;
    if (vt == SPREG_BF16 && bt == SPREG_BF16 && ct == SPREG_BF16) return COMBO_BF16_BF16OUT;
    if (vt == SPREG_F16 && bt == SPREG_F16 && ct == SPREG_F32) return COMBO_F16_F32OUT;
    return -1;
}

bool aligned(const void *p, size_t bytes) { return (reinterpret_cast<uintptr_t>(p) % bytes) == 0; }

template <int MR>
cudaError_t launch_combo(const ExecParams &p, int nv, int combo, dim3 grid, int threads, cudaStream_t s) {
    switch (combo) {
    case COMBO_F32: return launch_exec<MR, COMBO_F32>(p, nv, grid, threads, s);
    case COMBO_BF16_F32OUT: return launch_exec<MR, COMBO_BF16_F32OUT>(p, nv, grid, threads, s);
    case COMBO_BF16_BF16OUT: return launch_exec<MR, COMBO_BF16_BF16OUT>(p, nv, grid, threads, s);
    case COMBO_F16_F32OUT: return launch_exec<MR, COMBO_F16_F32OUT>(p, nv, grid, threads, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_mr(int mr, const ExecParams &p, int nv, int combo, dim3 grid, int threads, cudaStream_t s) {
    switch (mr) {
    case 2: return launch_combo<2>(p, nv, combo, grid, threads, s);
    case 4: return launch_combo<4>(p, nv, combo, grid, threads, s);
    case 6: return launch_combo<6>(p, nv, combo, grid, threads, s);
    case 8: return launch_combo<8>(p, nv, combo, grid, threads, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int MR>
cudaError_t launch_combo_batch(const BatchParams &p, int nv, int combo, unsigned grid, int threads, size_t smem,
                               cudaStream_t s) {
    switch (combo) {
    case COMBO_F32: return launch_exec_batch<MR, COMBO_F32>(p, nv, grid, threads, smem, s);
    case COMBO_BF16_F32OUT: return launch_exec_batch<MR, COMBO_BF16_F32OUT>(p, nv, grid, threads, smem, s);
    case COMBO_BF16_BF16OUT: return launch_exec_batch<MR, COMBO_BF16_BF16OUT>(p, nv, grid, threads, smem, s);
    case COMBO_F16_F32OUT: return launch_exec_batch<MR, COMBO_F16_F32OUT>(p, nv, grid, threads, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_mr_batch(int mr, const BatchParams &p, int nv, int combo, unsigned grid, int threads, size_t smem,
                            cudaStream_t s) {
    switch (mr) {
    case 2: return launch_combo_batch<2>(p, nv, combo, grid, threads, smem, s);
    case 4: return launch_combo_batch<4>(p, nv, combo, grid, threads, smem, s);
    case 6: return launch_combo_batch<6>(p, nv, combo, grid, threads, smem, s);
    case 8: return launch_combo_batch<8>(p, nv, combo, grid, threads, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int MR>
cudaError_t launch_combo_tile(const TileParams &p, int nv, bool gen, int combo, unsigned grid, int threads, size_t smem,
                              cudaStream_t s) {
    switch (combo) {
    case COMBO_F32: return launch_exec_tile<MR, COMBO_F32>(p, nv, gen, grid, threads, smem, s);
    case COMBO_BF16_F32OUT: return launch_exec_tile<MR, COMBO_BF16_F32OUT>(p, nv, gen, grid, threads, smem, s);
    case COMBO_BF16_BF16OUT: return launch_exec_tile<MR, COMBO_BF16_BF16OUT>(p, nv, gen, grid, threads, smem, s);
    case COMBO_F16_F32OUT: return launch_exec_tile<MR, COMBO_F16_F32OUT>(p, nv, gen, grid, threads, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_mr_tile(int mr, const TileParams &p, int nv, bool gen, int combo, unsigned grid, int threads,
                           size_t smem, cudaStream_t s) {
    switch (mr) {
    case 2: return launch_combo_tile<2>(p, nv, gen, combo, grid, threads, smem, s);
    case 4: return launch_combo_tile<4>(p, nv, gen, combo, grid, threads, smem, s);
    case 6: return launch_combo_tile<6>(p, nv, gen, combo, grid, threads, smem, s);
    case 8: return launch_combo_tile<8>(p, nv, gen, combo, grid, threads, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

// ------------------------------------------------------------------ per-device facts
struct DevFacts {
    int sms = 0;
    int smem_optin = 0;
    int smem_per_sm = 0;
    int *status = nullptr;     // status word of bounded waits
    int *counters = nullptr;   // work counters handed out round robin, one per launch
    int *flags = nullptr;      // load-balance flags, handed out round robin in blocks
};
constexpr int kCounters = 4096;
// Flags of the load-balanced splits, handed out round robin in blocks: a block is reused only
// after the pool has gone round (at least kLbFlags / kLbMaxBlock launches later), as the work
// counters are after kCounters launches.
constexpr int kLbFlags = 1 << 20;
constexpr int kLbMaxBlock = 1 << 14;  // flags of one launch's splits at most

namespace {
DevFacts g_facts[64];
std::mutex g_facts_mu;
}  // namespace

int dev_facts(DevFacts **out) {
    DevFacts *const facts = g_facts;
    std::mutex &mu = g_facts_mu;
    int dev = 0;
    SPREG_CUDA(cudaGetDevice(&dev));
    SPREG_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(mu);
    DevFacts &f = facts[dev];
    if (!f.status) {
        SPREG_CUDA(cudaDeviceGetAttribute(&f.sms, cudaDevAttrMultiProcessorCount, dev));
        SPREG_CUDA(cudaDeviceGetAttribute(&f.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        SPREG_CUDA(cudaDeviceGetAttribute(&f.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        if (f.smem_optin > kMaxSmem) f.smem_optin = kMaxSmem;
        int *buf = nullptr;
        SPREG_CUDA(cudaMalloc(&buf, sizeof(int) * (1 + kCounters + kLbFlags)));
        SPREG_CUDA(cudaMemset(buf, 0, sizeof(int) * (1 + kCounters + kLbFlags)));
        f.status = buf;
        f.counters = buf + 1;
        f.flags = buf + 1 + kCounters;
    }
    *out = &f;
    return SPREG_OK;
}

// Device status word of the current device (set-up on first use), for kernels outside this file.
int *device_status_word(int *st) {
    DevFacts *f;
    *st = dev_facts(&f);
    return *st ? nullptr : f->status;
}

int *next_counter(DevFacts *f) {
    static std::atomic<unsigned> next{0};
    return f->counters + (next.fetch_add(1) % kCounters);
}

// A block of n contiguous load-balance flags (n <= kLbMaxBlock), round robin as the counters: its
// offset in f->flags.
int32_t next_flags(int64_t n) {
    static std::atomic<unsigned long long> next{0};
    unsigned long long off = next.fetch_add((unsigned long long)n) % kLbFlags;
    if (off + (unsigned long long)n > (unsigned long long)kLbFlags) off = 0;
    return (int32_t)off;
}

// Self-test of the bounded waits: one CTA waits on an mbarrier that nothing arrives on, with a
// limit of `limit` polls, exactly as the executors wait on their stages.  The wait gives up, records
// kSelftestWaitCode in the device status word and the kernel returns; *polled receives how many polls
// were made (the limit).
constexpr int kSelftestWaitCode = 30;
__global__ void selftest_wait_kernel(int *status, uint32_t limit, uint32_t *polled) {
    __shared__ __align__(8) unsigned long long bar;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
    const bool ok = mbar_wait_bounded(b, 0, status, kSelftestWaitCode, limit);
    if (threadIdx.x == 0) *polled = ok ? 0u : limit;
}

int selftest_wait_impl(uint32_t limit, int32_t *status_out, uint32_t *polled_out, cudaStream_t stream) {
    SPREG_CHECK_ARG(status_out && polled_out, "null output");
    SPREG_CHECK_ARG(limit >= 1 && limit <= (1u << 22), "limit must be in [1, 2^22]");
    DevFacts *f;
    int st = dev_facts(&f);
    if (st) return st;
    uint32_t *polled = nullptr;
    SPREG_CUDA(cudaMallocAsync(&polled, sizeof(uint32_t), stream));
    selftest_wait_kernel<<<1, 32, 0, stream>>>(f->status, limit, polled);
    cudaError_t e = cudaGetLastError();
    int32_t v = 0;
    uint32_t p = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&p, polled, sizeof p, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&v, f->status, sizeof v, cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(polled, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "selftest: %s", cudaGetErrorString(e));
    *status_out = v;
    *polled_out = p;
    return SPREG_OK;
}

int noalloc_status_word(int dev, int32_t *v, int reset, bool *have);  // noalloc.cu

// The device's status word: the regular executors' word, or (when that is 0) the no-allocation
// entry point's.  A caller that has only used the no-allocation entry point on this device gets its
// word without the regular executors' per-device pool being created.
int device_status_impl(int32_t *status, int reset) {
    int dev = 0;
    SPREG_CUDA(cudaGetDevice(&dev));
    SPREG_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
    int32_t v_na = 0;
    bool have_na = false;
    int st = noalloc_status_word(dev, &v_na, reset, &have_na);
    if (st) return st;
    bool pool = false;
    {
        std::lock_guard<std::mutex> lk(g_facts_mu);
        pool = g_facts[dev].status != nullptr;
    }
    if (have_na && !pool) {
        if (status) *status = v_na;
        return SPREG_OK;
    }
    DevFacts *f;
    st = dev_facts(&f);
    if (st) return st;
    int v = 0;
    SPREG_CUDA(cudaMemcpy(&v, f->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (reset) SPREG_CUDA(cudaMemset(f->status, 0, sizeof(int)));
    if (status) *status = v ? v : v_na;
    return SPREG_OK;
}

// Columns per lane (strip width / 32) chosen automatically: wide strips amortise the per-entry
// index and value loads over more columns, narrow strips give more items when the launch is small.
// `others1` = the (panel, 32-column strip) items of the other SpMMs that share the launch, so a
// small SpMM in a large batch keeps wide strips.
int auto_nv(int64_t n, int64_t panels, int sms, int64_t others1) {
    int nv = 1;
    if (n >= 64) nv = 2;
    if (n >= 128) nv = 4;
    while (nv > 1 && panels * (n / (32 * nv)) + others1 / nv < (int64_t)sms * 8) nv >>= 1;
    return nv;
}

int64_t strip_items1(const spreg_packed *a, const spreg_exec_args *args) {
    return (a && args) ? a->info.num_panels * (args->n / 32) : 0;
}

// ------------------------------------------------------------------ one call -> problems
// Largest B tile (K tile rows x strip bytes) the shared-memory B kernel stages per stage.
constexpr int64_t kTileMaxStageB = 96 * 1024;

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Tensor map of B for the tile kernel: columns [0, cols) x rows [0, rows), a box of box_cols x
// box_rows elements, zeros outside.
int encode_b_map(CUtensorMap *map, const void *b, int dtype, int64_t cols, int64_t rows, int64_t ldb, int box_cols,
                 int box_rows) {
    auto enc = tensor_map_encoder();
    SPREG_CHECK_ARG(enc, "cuTensorMapEncodeTiled is not available from the driver");
    const CUtensorMapDataType t = dtype == SPREG_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                 : dtype == SPREG_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                       : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(ldb * (int64_t)dtype_bytes(dtype))};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, t, 2, const_cast<void *>(b), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SPREG_CHECK_ARG(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d) for B of %lld x %lld, ldb %lld", (int)r,
                    (long long)rows, (long long)cols, (long long)ldb);
    return SPREG_OK;
}

struct CallPlan {
    int mr, combo, nv;
    bool stream_kernel;      // run exec_kernel (register streams) instead of the batch kernel
    bool tile;               // run exec_tile_kernel (B tiles in shared memory)
    XProblem main, tail;     // whole strips (NV) and the NV = 1 remainder
    TProblem tmain, ttail;   // the same problems for exec_tile_kernel
    int64_t stage_b_main, stage_b_tail;
    bool has_main, has_tail;
    int64_t xbuf;            // per-warp buffer for this pack
    ExecParams sp;           // parameters of the register-stream kernel
    int warps;
    int warps_req;           // warps_per_cta as asked (0: each kernel's own choice) -- the CTA tiling
    int rounds;              // panel rounds of the B-tile kernel (1: B tiles in the ring stages)
    // Load balance: work-order positions [0, lb_heavy) run K tiles [0, lb_split) into C (the low
    // half), and [lb_split, T) from zero (the high half), which adds into C once the low half of its
    // (panel, strip) is stored; flags of the main and tail problems at these offsets of f->flags.
    int64_t lb_heavy = 0;
    int32_t lb_split = 0;
    int32_t lb_flags_main = 0, lb_flags_tail = 0;
    const spreg_packed *a = nullptr;
    const spreg_exec_args *args = nullptr;
};

// The load-balanced split of a pack run by the B-tile kernel with W panels per job and S strips:
// the launch has ceil(P / W) x S jobs (+ other_jobs of other SpMMs).  When that leaves SMs idle, the
// heaviest job groups (whole groups of W panels in work order, as long as their first panel's work
// estimate exceeds half the heaviest one's) are split at K tile T / 2, each split group adding S
// jobs, until the idle SMs are used, unless the first unsplit group is within a fifth of the
// heaviest.  That shortens the longest jobs of a launch with about one job per SM (a single SpMM);
// a launch with a full wave of jobs or more is balanced by the work counter already and is not
// split.
void balance_of(const spreg_packed *a, int W, int64_t S, int64_t slots, int64_t other_jobs, int64_t *heavy,
                int32_t *split) {
    *heavy = 0;
    *split = 0;
    const int64_t P = a->geom.P, T = a->geom.T;
    if (T < 2 || P < 2 || W < 1 || S < 1 || a->list_packed || (int64_t)a->work_desc.size() != P ||
        a->work_desc[0] <= 0)
        return;
    const int64_t groups = (P + W - 1) / W;
    const int64_t free_slots = slots - groups * S - other_jobs;
    const int64_t top = a->work_desc[0];
    int64_t g = 0;
    while (g < groups && (g + 1) * S <= free_slots && 2 * a->work_desc[(size_t)(g * W)] > top) ++g;
    if (g == 0) return;
    // the longest job after the split is the first unsplit group's (or half the heaviest one's): skip a
    // split that would shorten it by less than a fifth (the combine and the scratch cost more)
    if (g < groups && 5 * a->work_desc[(size_t)(g * W)] > 4 * top) return;
    // a split of some groups only pays (the general kernel form, the combine) when the heaviest
    // panels are a real tail: at least twice the median panel's work (measured on 2048 x 512 @ 90 %,
    // M_r = 4: a tail of 1.8x ran 0.96x, one of 3.0x 1.2x); splitting every group doubles the jobs
    if (g < groups && top < 2 * a->work_desc[(size_t)(P / 2)]) return;
    if (std::min<int64_t>(g * W, P) * S > kLbMaxBlock) return;  // one flag per split (panel, strip)
    *heavy = std::min<int64_t>(g * W, P);
    *split = (int32_t)(T / 2);
}

// Consumer warps (panels per job) of the B-tile kernel for a call: as asked, else 15.
int tile_warps_of(const spreg_exec_args *args) {
    return args->warps_per_cta > 0 ? std::min(args->warps_per_cta, kTileMaxWarps) : kTileMaxWarps;
}

int plan_call(const spreg_packed *a, const spreg_exec_args *args, CallPlan *cp, int64_t others1) {
    SPREG_CHECK_ARG(a && args, "null packed matrix or args");
    const spreg_packed_info &in = a->info;
    const int combo = combo_of(in.value_dtype, args->b_dtype, args->c_dtype);
    SPREG_CHECK_ARG(combo >= 0, "unsupported dtype combination values=%d B=%d C=%d (B must match the values; "
                    "C is F32, or BF16 for BF16 values)", in.value_dtype, args->b_dtype, args->c_dtype);
    SPREG_CHECK_ARG(args->n >= 0, "n must be >= 0");
    SPREG_CHECK_ARG(args->n == 0 || in.rows == 0 || (args->c && (args->b || in.cols == 0)), "null B or C");
    SPREG_CHECK_ARG(args->ldb >= args->n || in.cols == 0, "ldb (%lld) < n (%lld)", (long long)args->ldb,
                    (long long)args->n);
    SPREG_CHECK_ARG(args->ldc >= args->n, "ldc (%lld) < n (%lld)", (long long)args->ldc, (long long)args->n);
    SPREG_CHECK_ARG(args->epilogue == SPREG_EPILOGUE_NONE || args->epilogue == SPREG_EPILOGUE_RELU, "bad epilogue");
    SPREG_CHECK_ARG(args->meta_staging >= 0 && args->meta_staging <= 2, "meta_staging must be 0, 1 or 2");
    SPREG_CHECK_ARG(args->b_staging >= 0 && args->b_staging <= 2, "b_staging must be 0, 1 or 2");
    SPREG_CHECK_ARG(args->job_order == 0 || args->job_order == 1, "job_order must be 0 or 1");
    SPREG_CHECK_ARG(args->panel_rounds >= 0 && args->panel_rounds <= kTileMaxRounds, "panel_rounds must be in [0, %d]",
                    kTileMaxRounds);
    const int rounds = args->panel_rounds > 1 ? args->panel_rounds : 1;
    SPREG_CHECK_ARG(args->load_balance == 0 || args->load_balance == 1, "load_balance must be 0 or 1");
    SPREG_CHECK_ARG(args->load_balance == 0 ||
                        (args->c_dtype == SPREG_F32 && in.value_dtype != SPREG_F16 && args->b_staging != 2 &&
                         args->meta_staging != 2),
                    "load_balance needs FP32 C, FP32 or BF16 values and the B-tile kernel (b_staging 0 or 1)");
    SPREG_CHECK_ARG(rounds == 1 || (args->b_staging != 2 && args->meta_staging != 2),
                    "panel_rounds > 1 runs the shared-memory B-tile kernel (b_staging 0 or 1, meta_staging 0 or 1)");
    int dev = -1;
    SPREG_CUDA(cudaGetDevice(&dev));
    SPREG_CHECK_ARG(dev == a->device, "packed matrix lives on device %d, current device is %d", a->device, dev);
    DevFacts *f;
    int st = dev_facts(&f);
    if (st) return st;
    int nv;
    switch (args->nr) {
    case 0: nv = auto_nv(args->n, in.num_panels, f->sms, others1); break;
    case 32: nv = 1; break;
    case 64: nv = 2; break;
    case 128: nv = 4; break;
    // 256 and 512: wide strips where a kernel has them (below: the B-tile kernel with 16-bit B, the
    // gather kernel with FP32), else 128
    case 256: nv = 4; break;
    case 512: nv = 4; break;
    default: SPREG_FAIL(SPREG_ERR_INVALID_ARG, "nr must be 0, 32, 64, 128, 256 or 512 (got %d)", args->nr);
    }
    const size_t bsz = dtype_bytes(args->b_dtype), csz = dtype_bytes(args->c_dtype);
    while (nv > 1 && !(aligned(args->b, bsz * nv) && args->ldb % nv == 0 && aligned(args->c, csz * nv) &&
                       args->ldc % nv == 0))
        nv >>= 1;
    cp->mr = in.mr;
    cp->combo = combo;
    cp->warps = args->warps_per_cta > 0 ? args->warps_per_cta : 4;
    cp->warps_req = args->warps_per_cta > 0 ? args->warps_per_cta : 0;
    SPREG_CHECK_ARG(cp->warps >= 1 && cp->warps <= 8, "warps_per_cta must be in [1, 8]");
    cp->xbuf = (a->max_exec_bytes + 127) / 128 * 128;
    const bool x_fits = a->exec && 1024 + 2 * cp->xbuf <= f->smem_optin;
    SPREG_CHECK_ARG(args->meta_staging != 1 || x_fits, "the execution-layout kernel cannot run this pack "
                    "(largest block %lld bytes)", (long long)a->max_exec_bytes);
    cp->stream_kernel = args->meta_staging == 2 || !x_fits;

    // Shared-memory B tiles: one copy per K tile row of the strip's columns (16-byte aligned rows,
    // reads rounded up to 16 bytes stay inside each row of B), a tile that fits a stage, and the
    // column ranges of K tiles (not the per-panel offsets of panel-by-panel packs).
    const int64_t kt_rows = a->geom.kt;
    const int box_rows = (int)std::min<int64_t>(kt_rows, kTileBoxRows);
    const int64_t staged_rows = (kt_rows + box_rows - 1) / box_rows * box_rows;
    auto tile_rows_ok = [&](int nvv) { return staged_rows * 32 * nvv * (int64_t)bsz <= kTileMaxStageB; };
    const bool tile_base_ok = a->exec && !a->list_packed && aligned(args->b, 16) &&
                              (args->ldb * (int64_t)bsz) % 16 == 0 && 1024 + 2 * cp->xbuf <= f->smem_optin;
    // Panel rounds keep the strip of every K tile resident: T tiles of staged_rows rows each.
    auto strip_bytes = [&](int nvv) { return (a->geom.T * staged_rows * 32 * nvv * (int64_t)bsz + 127) / 128 * 128; };
    auto strip_fits = [&](int nvv) { return 1024 + strip_bytes(nvv) + 2 * cp->xbuf <= f->smem_optin; };
    cp->rounds = rounds;
    if (rounds > 1) {
        SPREG_CHECK_ARG(tile_base_ok, "panel rounds need a dense/CSR pack, a 16-byte aligned B with 16-byte aligned "
                        "rows, and execution blocks that fit shared memory");
        SPREG_CHECK_ARG(args->n <= INT32_MAX && a->geom.T < 65536, "panel rounds: n or the K tile count out of range");
        if (args->nr == 0)
            while (nv > 1 && !strip_fits(nv)) nv >>= 1;
        SPREG_CHECK_ARG(strip_fits(nv) && strip_fits(1),
                        "panel rounds: the strip of B for all K tiles (%lld bytes at %d columns) does not fit shared "
                        "memory; use a narrower strip (nr) or panel_rounds 0", (long long)strip_bytes(nv), 32 * nv);
    }
    if (args->b_staging == 1) {
        SPREG_CHECK_ARG(tile_base_ok, "shared-memory B tiles need a dense/CSR pack, a 16-byte aligned B with "
                        "16-byte aligned rows, and execution blocks that fit shared memory");
        SPREG_CHECK_ARG(args->meta_staging != 2, "b_staging = 1 runs the execution-layout metadata path");
        SPREG_CHECK_ARG(args->n <= INT32_MAX, "n out of range for shared-memory B tiles");
    }

    // Wide strips for 16-bit B in the B-tile kernel: NV = 8 (256 columns, one 16-byte shared-memory
    // load per lane and entry) spreads each entry's index and value loads over twice the columns.
    // Taken when that kernel runs, the stage still holds 64 KB, the launch keeps enough
    // (panel, strip) items, and at least 85 % of the entries are in groups with their own loop there
    // (the single rows and the all-rows kernel; other patterns dispatch per half step, slower than
    // NV = 4 where they are common: BF16 2048 x 512 at 70-80 % sparsity) -- or when nr = 256 asks.
    int64_t hot = 0, all = 0;
    for (int i = 0; i < in.num_nkern; ++i) {
        const int p = a->id_to_pattern[i];
        all += a->id_entries[i];
        if ((p & (p - 1)) == 0 || p == (1 << in.mr) - 1) hot += a->id_entries[i];
    }
    const bool hot_set = all > 0 && 100 * hot >= 85 * all;
    // load balance: K-tiled packs run the B-tile kernel; the split itself is decided below, once
    // the strip width is known
    const bool lb = args->load_balance && a->geom.T >= 2 && !a->list_packed;
    SPREG_CHECK_ARG(!lb || (tile_base_ok && args->n <= INT32_MAX),
                    "load_balance: the B-tile kernel cannot run this call (a 16-byte aligned B with 16-byte "
                    "aligned rows is needed)");
    const bool tile_kernel =
        args->b_staging == 1 || rounds > 1 || lb || (args->b_staging == 0 && tile_base_ok && args->meta_staging != 2 &&
                                 !cp->stream_kernel && a->geom.T > 1 && args->n <= INT32_MAX &&
                                 staged_rows * 32 * nv * (int64_t)bsz <= 64 * 1024);
    if (tile_kernel && bsz == 2 && in.mr <= 4 && nv == 4 && (args->nr == 0 || args->nr >= 256) && args->n >= 256 &&
        (rounds == 1 || strip_fits(8)) &&
        staged_rows * 256 * (int64_t)bsz <= 64 * 1024 && aligned(args->b, 16) && args->ldb % 8 == 0 &&
        aligned(args->c, csz * 8) && args->ldc % 8 == 0 &&
        (args->nr >= 256 || (hot_set && in.num_panels * (args->n / 256) + others1 / 8 >= (int64_t)f->sms * 8)))
        nv = 8;
    // Wide FP32 strips in the gather kernel (nr = 256: NV = 8; nr = 512 and M_r <= 4: NV = 16), lanes
    // interleaved by 16-byte quarters: at high sparsity an entry's index, value and address work is
    // shared by 8 or 16 columns a lane.  Whole strips only; columns past the last one run as the
    // 32-column tail launch.
    const bool gather_wide = (args->nr == 256 || args->nr == 512) && !tile_kernel && !cp->stream_kernel &&
                             combo == COMBO_F32 && nv == 4 && args->n >= 256 && aligned(args->b, 16) &&
                             args->ldb % 4 == 0 && aligned(args->c, 16) && args->ldc % 4 == 0;
    if (gather_wide) nv = args->nr == 512 && in.mr <= 4 && args->n >= 512 ? 16 : 8;
    // 16-bit B in the gather kernel at M_r <= 4: 256-column strips (NV = 8, one 16-byte load of 8
    // columns a lane and entry, the mixed-precision FMA of the B-tile kernel's wide strips), and
    // for nr = 512 512-column strips (NV = 16: 8 columns a lane in each 256-column half)
    const bool gather_wide16 = (args->nr == 256 || args->nr == 512) && !tile_kernel && !cp->stream_kernel &&
                               bsz == 2 && in.mr <= 4 && nv == 4 && args->n >= 256 && aligned(args->b, 16) &&
                               args->ldb % 8 == 0 && aligned(args->c, csz * 8) && args->ldc % 8 == 0;
    if (gather_wide16) nv = args->nr == 512 && args->n >= 512 ? 16 : 8;
    cp->nv = nv;
    const int64_t n_main = (args->n / (32 * nv)) * (32 * nv);
    int64_t lb_heavy = 0;
    int32_t lb_split = 0;
    if (lb) {
        const int64_t strips = args->n % nv == 0 ? (args->n + 32 * nv - 1) / (32 * nv)
                                                 : n_main / (32 * nv) + (args->n - n_main + 31) / 32;
        const int W = tile_warps_of(args) * rounds;  // panels per job
        // other SpMMs of the launch: their (panel, 32-column) items over W panels and 4 columns a job
        balance_of(a, W, strips, f->sms, others1 / ((int64_t)W * 4), &lb_heavy, &lb_split);
    }

    XProblem base = {};
    base.exec = a->exec;
    base.exec_offs = a->exec_offs;
    base.panel_rank = a->panel_rank;
    base.scales = a->scales;
    base.B = args->b;
    base.C = args->c;
    base.ldb = args->ldb;
    base.ldc = args->ldc;
    base.M = in.rows;
    base.P = (int32_t)a->geom.P;
    base.T = (int32_t)a->geom.T;
    base.ppt = (int32_t)a->geom.ppt;
    base.load_c = args->load_c ? 1 : 0;
    base.epilogue = args->epilogue;
    base.order = args->job_order;
    cp->has_main = n_main > 0 && base.P > 0;
    cp->has_tail = args->n > n_main && base.P > 0;
    cp->main = base;
    cp->main.col_begin = 0;
    cp->main.col_end = n_main;
    cp->main.S = (int32_t)(n_main / (32 * nv));
    cp->tail = base;
    cp->tail.col_begin = n_main;
    cp->tail.col_end = args->n;
    cp->tail.S = (int32_t)((args->n - n_main + 31) / 32);

    cp->tile = false;
    // b_staging = 0 picks the tile kernel for K-tiled packs whose stage leaves room for all 16
    // consumer warps (64 KB of B per stage): measured faster than the gather kernel there (FP32,
    // 2048 x 512 @ 90 %, K_c = 128: 13.2 vs 13.8 us per SpMM).  It never fails in that mode.
    const bool auto_tile = args->b_staging == 0 && !gather_wide && !gather_wide16 && tile_base_ok &&
                           args->meta_staging != 2 &&
                           !cp->stream_kernel && a->geom.T > 1 && args->n <= INT32_MAX &&
                           staged_rows * 32 * nv * (int64_t)bsz <= 64 * 1024;
    if (args->b_staging == 1 || rounds > 1 || lb || auto_tile) {
        const bool main_ok = !cp->has_main || rounds > 1 || tile_rows_ok(nv);
        const bool tail_ok = !cp->has_tail || rounds > 1 || tile_rows_ok(1);
        SPREG_CHECK_ARG(main_ok && tail_ok, "shared-memory B tiles: a K tile of %lld rows x %d columns exceeds a "
                        "stage (%lld bytes); pack with a smaller k_tile", (long long)kt_rows, 32 * nv,
                        (long long)kTileMaxStageB);
        cp->tile = true;
        cp->stream_kernel = false;
        TProblem tb = {};
        tb.exec = a->exec;
        tb.exec_offs = a->exec_offs;
        tb.panel_order = a->panel_order;
        tb.scales = a->scales;
        tb.B = args->b;
        tb.C = args->c;
        tb.ldb = args->ldb;
        tb.ldc = args->ldc;
        SPREG_CHECK_ARG(in.rows <= INT32_MAX && a->geom.T < 32768, "shared-memory B tiles: too many rows or K tiles");
        tb.M = (int32_t)in.rows;
        tb.P = (int32_t)a->geom.P;
        tb.T = (int32_t)a->geom.T;
        tb.combine = 0;
        tb.pad16 = 0;
        tb.flag_off = 0;
        tb.load_c = args->load_c ? 1 : 0;
        tb.epilogue = (int16_t)args->epilogue;
        tb.order = (int16_t)args->job_order;
        tb.kt = (int32_t)kt_rows;
        tb.col_offset = (int32_t)in.col_offset;
        tb.box_rows = (int16_t)box_rows;
        tb.t_begin = 0;
        tb.t_end = (int16_t)a->geom.T;
        tb.pos_begin = 0;
        tb.count = (int32_t)a->geom.P;
        cp->lb_heavy = lb_heavy;
        cp->lb_split = lb_split;
        cp->a = a;
        cp->args = args;
        const int64_t brows = in.col_offset + a->geom.K;
        // Columns past the last whole strip: when n is a multiple of NV they run as one more strip of
        // the main problem, masked per lane (B tiles past column n are zero-filled by the tensor copy;
        // lanes whose columns start at or past n store nothing), inside the same launch.  Else (the
        // lanes' NV-column stores would cross n) as 32-column strips of their own launch.
        const bool merge_tail = cp->has_tail && args->n % nv == 0;
        const int64_t n_tile_main = merge_tail ? args->n : n_main;
        if (merge_tail) {
            cp->has_main = true;
            cp->has_tail = false;
        }
        cp->tmain = tb;
        cp->tmain.col_begin = 0;
        cp->tmain.col_end = (int32_t)n_tile_main;
        cp->tmain.S = (int32_t)((n_tile_main + 32 * nv - 1) / (32 * nv));
        if (cp->has_main && (st = encode_b_map(&cp->tmain.tmap, args->b, args->b_dtype, n_tile_main, brows, args->ldb,
                                               32 * nv, box_rows)))
            return st;
        cp->ttail = tb;
        cp->ttail.col_begin = (int32_t)n_main;
        cp->ttail.col_end = (int32_t)args->n;
        cp->ttail.S = cp->tail.S;
        if (cp->has_tail && (st = encode_b_map(&cp->ttail.tmap, args->b, args->b_dtype, args->n, brows, args->ldb, 32,
                                               box_rows)))
            return st;
        cp->stage_b_main = rounds > 1 ? strip_bytes(nv) : (staged_rows * 32 * nv * (int64_t)bsz + 127) / 128 * 128;
        cp->stage_b_tail = rounds > 1 ? strip_bytes(1) : (staged_rows * 32 * (int64_t)bsz + 127) / 128 * 128;
    }

    ExecParams &p = cp->sp;
    p = ExecParams{};
    p.arena = a->arena;
    p.descs = a->descs;
    p.scales = a->scales;
    p.B = args->b;
    p.C = args->c;
    p.ldb = args->ldb;
    p.ldc = args->ldc;
    p.M = in.rows;
    p.N = args->n;
    p.P = a->geom.P;
    p.ppt = a->geom.ppt;
    p.T = a->geom.T;
    p.nk = in.num_nkern;
    p.load_c = args->load_c ? 1 : 0;
    p.epilogue = args->epilogue;
    p.status = f->status;
    for (int i = 0; i < 256; ++i) p.id_pattern[i] = a->id_to_pattern[i];
    return SPREG_OK;
}

// Register-stream kernel for one call: NV launch over whole strips, NV = 1 launch for the rest.
int launch_stream(const CallPlan &cp, cudaStream_t stream) {
    const unsigned gx = (unsigned)((cp.sp.P + cp.warps - 1) / cp.warps);
    const int threads = 32 * cp.warps;
    if (cp.has_main) {
        ExecParams p = cp.sp;
        p.col_begin = 0;
        const int64_t gy = cp.main.S;
        SPREG_CHECK_ARG(gy <= 65535, "n too large for one launch");
        cudaError_t e = launch_mr(cp.mr, p, cp.nv, cp.combo, dim3(gx, (unsigned)gy), threads, stream);
        if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "executor launch: %s", cudaGetErrorString(e));
    }
    if (cp.has_tail) {
        ExecParams p = cp.sp;
        p.col_begin = cp.tail.col_begin;
        const int64_t gy = cp.tail.S;
        SPREG_CHECK_ARG(gy <= 65535, "n too large for one launch");
        cudaError_t e = launch_mr(cp.mr, p, 1, cp.combo, dim3(gx, (unsigned)gy), threads, stream);
        if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "executor launch: %s", cudaGetErrorString(e));
    }
    return SPREG_OK;
}

// One batch-kernel launch per group of at most kMaxBatchProblems problems of one configuration.
struct Group {
    int mr, combo, nv;
    int warps_req = 0;  // warps per CTA asked by the first call that asked (0: 8)
    std::vector<XProblem> probs;
    int64_t xbuf = 0;
};

int launch_groups(std::map<std::tuple<int, int, int>, Group> &groups, cudaStream_t stream) {
    DevFacts *f;
    int st = dev_facts(&f);
    if (st) return st;
    for (auto &kv : groups) {
        Group &g = kv.second;
        for (size_t first = 0; first < g.probs.size(); first += kMaxBatchProblems) {
            const size_t cnt = std::min<size_t>(kMaxBatchProblems, g.probs.size() - first);
            BatchParams bp;
            bp.nprob = (int32_t)cnt;
            int64_t items = 0;
            for (size_t i = 0; i < cnt; ++i) {
                bp.prob[i] = g.probs[first + i];
                bp.prob[i].item_begin = items;
                items += (int64_t)bp.prob[i].P * bp.prob[i].S;
            }
            if (items == 0) continue;
            SPREG_CHECK_ARG(items <= INT32_MAX, "too many work items in one launch");
            bp.items = items;
            bp.xbuf = (int32_t)g.xbuf;
            bp.status = f->status;
            bp.counter = next_counter(f);
            // warps per CTA: as asked, else 8; fewer if the buffers do not fit
            int nw = g.warps_req > 0 ? g.warps_req : 8;
            if (g.nv >= 8 && g.combo == COMBO_F32) nw = std::min(nw, kWideMaxWarps);  // the kernel's bound
            while (nw > 1 && 1024 + 2 * g.xbuf * nw > f->smem_optin) nw >>= 1;
            const size_t smem = (size_t)(1024 + 2 * g.xbuf * nw);
            const int threads = 32 * nw;
            const int per_sm = std::max(1, std::min((int)(f->smem_per_sm / (int64_t)smem), 2048 / threads));
            const int64_t ctas = std::min<int64_t>((int64_t)f->sms * per_sm, (items + nw - 1) / nw);
            SPREG_CUDA(cudaMemsetAsync(bp.counter, 0, sizeof(int), stream));
            cudaError_t e = launch_mr_batch(g.mr, bp, g.nv, g.combo, (unsigned)ctas, threads, smem, stream);
            if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "batched executor launch: %s", cudaGetErrorString(e));
        }
    }
    return SPREG_OK;
}

// One tile-kernel launch per group of at most kMaxBatchProblems problems of one configuration.
struct TileGroup {
    int mr, combo, nv, rounds;
    bool gen = false;  // the kernel's general form: panel rounds, K-tile / position ranges, split halves
    int warps_req = 0;  // consumer warps (panels per job) asked by the first call that asked (0: 16)
    std::vector<TProblem> probs;
    int64_t xbuf = 0, stage_b = 0;
};

int launch_tile_groups(std::map<std::tuple<int, int, int, int, bool>, TileGroup> &groups, cudaStream_t stream) {
    DevFacts *f;
    int st = dev_facts(&f);
    if (st) return st;
    for (auto &kv : groups) {
        TileGroup &g = kv.second;
        // consumer warps: as asked, else 15; fewer if the stages do not fit.  With panel rounds: two
        // resident strips and four ring stages where they fit, else one strip (the producer then waits
        // for a job's last stage before loading the next job's strip) and two stages.
        const bool res = g.rounds > 1;
        int W = g.warps_req > 0 ? std::min(g.warps_req, kTileMaxWarps) : kTileMaxWarps;
        int nbuf = 0, stages = kTileStages;
        auto smem_of = [&](int w, int nb, int ns) {
            return res ? (int64_t)1024 + nb * g.stage_b + (int64_t)ns * w * g.xbuf
                       : (int64_t)1024 + kTileStages * (g.stage_b + (int64_t)w * g.xbuf);
        };
        auto pick = [&](int w) {
            if (!res) return smem_of(w, 0, kTileStages) <= f->smem_optin;
            const int cand[4][2] = {{2, kTileMaxStages}, {2, 2}, {1, kTileMaxStages}, {1, 2}};
            for (auto &c : cand)
                if (smem_of(w, c[0], c[1]) <= f->smem_optin) {
                    nbuf = c[0];
                    stages = c[1];
                    return true;
                }
            return false;
        };
        while (W > 1 && !pick(W)) W >>= 1;
        SPREG_CHECK_ARG(pick(W), "shared-memory B tiles: a stage does not fit (%lld bytes)",
                        (long long)smem_of(W, res ? 1 : 0, kTileStages));
        const size_t smem = (size_t)smem_of(W, nbuf, stages);
        const int threads = 32 * (W + 1);
        for (size_t first = 0; first < g.probs.size(); first += kTileMaxProblems) {
            const size_t cnt = std::min<size_t>(kTileMaxProblems, g.probs.size() - first);
            TileParams tp;
            tp.nprob = (int32_t)cnt;
            int64_t jobs = 0;
            for (size_t i = 0; i < cnt; ++i) {
                TProblem &pr = tp.prob[i];
                pr = g.probs[first + i];
                pr.job_begin = (int32_t)jobs;
                const int64_t per_job = (int64_t)W * g.rounds;
                jobs += (int64_t)((pr.count + per_job - 1) / per_job) * pr.S;
                if (jobs > INT32_MAX) break;
            }
            if (jobs == 0) continue;
            SPREG_CHECK_ARG(jobs <= INT32_MAX, "too many jobs in one launch");
            tp.jobs = jobs;
            tp.xbuf = (int32_t)g.xbuf;
            tp.warps = W;
            tp.stage_b = (int32_t)g.stage_b;
            tp.stages = stages;
            tp.rounds = g.rounds;
            tp.nbuf = nbuf;
            tp.pad_ = 0;
            tp.flags = f->flags;
            tp.status = f->status;
            tp.counter = next_counter(f);
            const int per_sm = std::max(1, std::min((int)(f->smem_per_sm / (int64_t)smem), 2048 / threads));
            const int64_t ctas = std::min<int64_t>((int64_t)f->sms * per_sm, jobs);
            SPREG_CUDA(cudaMemsetAsync(tp.counter, 0, sizeof(int), stream));
            cudaError_t e = launch_mr_tile(g.mr, tp, g.nv, g.gen, g.combo, (unsigned)ctas, threads, smem, stream);
            if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "tile executor launch: %s", cudaGetErrorString(e));
        }
    }
    return SPREG_OK;
}

void add_tile_call(std::map<std::tuple<int, int, int, int, bool>, TileGroup> &groups, const CallPlan &cp) {
    auto add = [&](const TProblem &pr, int nv, int64_t stage_b) {
        const bool gen = cp.rounds > 1 || cp.lb_heavy > 0;
        TileGroup &g = groups[std::make_tuple(cp.mr, cp.combo, nv, cp.rounds, gen)];
        g.mr = cp.mr;
        g.combo = cp.combo;
        g.nv = nv;
        g.rounds = cp.rounds;
        g.gen = gen;
        if (!g.warps_req) g.warps_req = cp.warps_req;
        g.probs.push_back(pr);
        g.xbuf = std::max(g.xbuf, cp.xbuf);
        g.stage_b = std::max(g.stage_b, stage_b);
    };
    auto add_split = [&](const TProblem &pr, int nv, int64_t stage_b, int32_t flag_off) {
        if (cp.lb_heavy <= 0) {
            add(pr, nv, stage_b);
            return;
        }
        // heavy panels: K tiles [0, split) into C (no epilogue; flags each (panel, strip) when stored),
        // then [split, T) from zero, added into C after the low half (the epilogue after the add).
        // The low halves' jobs come first in the launch, so a high half waits only on jobs that are
        // already running or done.
        TProblem lo = pr, hi = pr, rest = pr;
        lo.count = hi.count = (int32_t)cp.lb_heavy;
        lo.t_end = (int16_t)cp.lb_split;
        lo.epilogue = SPREG_EPILOGUE_NONE;
        lo.combine = 1;
        lo.flag_off = flag_off;
        hi.t_begin = (int16_t)cp.lb_split;
        hi.load_c = 0;
        hi.combine = 2;
        hi.flag_off = flag_off;
        add(lo, nv, stage_b);
        add(hi, nv, stage_b);
        if (cp.lb_heavy < pr.P) {
            rest.pos_begin = (int32_t)cp.lb_heavy;
            rest.count = pr.P - (int32_t)cp.lb_heavy;
            add(rest, nv, stage_b);
        }
    };
    if (cp.has_main) add_split(cp.tmain, cp.nv, cp.stage_b_main, cp.lb_flags_main);
    if (cp.has_tail) add_split(cp.ttail, 1, cp.stage_b_tail, cp.lb_flags_tail);
}

void add_call(std::map<std::tuple<int, int, int>, Group> &groups, const CallPlan &cp) {
    auto add = [&](const XProblem &pr, int nv) {
        Group &g = groups[std::make_tuple(cp.mr, cp.combo, nv)];
        g.mr = cp.mr;
        g.combo = cp.combo;
        g.nv = nv;
        if (!g.warps_req) g.warps_req = cp.warps_req;
        g.probs.push_back(pr);
        g.xbuf = std::max(g.xbuf, cp.xbuf);
    };
    if (cp.has_main) add(cp.main, cp.nv);
    if (cp.has_tail) add(cp.tail, 1);
}

int run_calls(const spreg_packed *const *as, const spreg_exec_args *const *args, int32_t n, cudaStream_t stream) {
    std::map<std::tuple<int, int, int>, Group> groups;
    std::map<std::tuple<int, int, int, int, bool>, TileGroup> tgroups;
    std::vector<CallPlan> streams;
    int64_t items1 = 0;
    for (int32_t i = 0; i < n; ++i) items1 += strip_items1(as[i], args[i]);
    std::vector<CallPlan> plans((size_t)n);
    DevFacts *f;
    int st = dev_facts(&f);
    if (st) return st;
    for (int32_t i = 0; i < n; ++i) {
        CallPlan &cp = plans[(size_t)i];
        st = plan_call(as[i], args[i], &cp, items1 - strip_items1(as[i], args[i]));
        if (st != SPREG_OK) return st;
        if (cp.lb_heavy > 0) {
            // one zeroed flag per split (panel, strip) of the main and the tail problem
            const int64_t nm = cp.has_main ? cp.lb_heavy * cp.tmain.S : 0;
            const int64_t nt = cp.has_tail ? cp.lb_heavy * cp.ttail.S : 0;
            cp.lb_flags_main = next_flags(nm + nt);
            cp.lb_flags_tail = cp.lb_flags_main + (int32_t)nm;
            SPREG_CUDA(cudaMemsetAsync(f->flags + cp.lb_flags_main, 0, (size_t)(nm + nt) * sizeof(int), stream));
        }
    }
    for (const CallPlan &cp : plans) {
        if (cp.tile) add_tile_call(tgroups, cp);
        else if (cp.stream_kernel) streams.push_back(cp);
        else add_call(groups, cp);
    }
    st = launch_groups(groups, stream);
    if (st == SPREG_OK) st = launch_tile_groups(tgroups, stream);
    for (size_t i = 0; i < streams.size() && st == SPREG_OK; ++i) st = launch_stream(streams[i], stream);
    return st;
}

int explain_impl(const spreg_packed *a, const spreg_exec_args *args, char *buf, int64_t len) {
    SPREG_CHECK_ARG(a && args && buf && len > 0, "null argument");
    CallPlan cp;
    int st = plan_call(a, args, &cp, 0);
    if (st != SPREG_OK) return st;
    const char *kernel = cp.tile ? "exec_tile_kernel" : cp.stream_kernel ? "exec_kernel" : "exec_batch_kernel";
    const int64_t n_main = cp.has_main ? (cp.tile ? (int64_t)cp.tmain.col_end : (int64_t)cp.main.col_end) : 0;
    snprintf(buf, (size_t)len,
             "kernel=%s mr=%d nv=%d strip_columns=%d main_columns=%lld tail_columns=%lld k_tiles=%lld k_tile=%lld "
             "warps=%d rounds=%d load_balance_heavy=%lld load_balance_split=%d",
             kernel, cp.mr, cp.nv, 32 * cp.nv, (long long)n_main, (long long)(cp.has_tail ? args->n - n_main : 0),
             (long long)a->geom.T, (long long)a->geom.kt, cp.tile ? tile_warps_of(args) : cp.warps, cp.rounds,
             (long long)cp.lb_heavy, cp.lb_split);
    return SPREG_OK;
}

int load_balance_plan_impl(const spreg_packed *a, const spreg_exec_args *args, int64_t *heavy, int32_t *split,
                           int32_t *ids, int64_t max_ids) {
    SPREG_CHECK_ARG(a && args && heavy && split, "null argument");
    CallPlan cp;
    spreg_exec_args x = *args;
    x.load_balance = 1;
    int st = plan_call(a, &x, &cp, 0);
    if (st != SPREG_OK) return st;
    *heavy = cp.lb_heavy;
    *split = cp.lb_split;
    if (ids)
        for (int64_t i = 0; i < *heavy && i < max_ids; ++i) ids[i] = a->order_host[(size_t)i];
    return SPREG_OK;
}

int execute_impl(const spreg_packed *a, const spreg_exec_args *args, cudaStream_t stream) {
    return run_calls(&a, &args, 1, stream);
}

int execute_timed_impl(const spreg_packed *a, const spreg_exec_args *args, int64_t num_runs, double *median_ns,
                       cudaStream_t stream) {
    SPREG_CHECK_ARG(median_ns, "null median_ns");
    SPREG_CHECK_ARG(num_runs >= 1, "num_runs must be >= 1");
    int st;
    const int kIters = 150;  // MEASURED_ITERATIONS of template:317
    for (int64_t r = 0; r < num_runs; ++r)
        if ((st = execute_impl(a, args, stream))) return st;
    std::vector<cudaEvent_t> ev(2 * kIters);
    for (auto &e : ev) SPREG_CUDA(cudaEventCreate(&e));
    st = SPREG_OK;
    for (int it = 0; it < kIters && !st; ++it) {
        cudaEventRecord(ev[2 * it], stream);
        for (int64_t r = 0; r < num_runs && !st; ++r) st = execute_impl(a, args, stream);
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
    if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "timed execute: %s", cudaGetErrorString(e));
    std::sort(t.begin(), t.end());
    *median_ns = (t[kIters / 2 - 1] + t[kIters / 2]) / 2.0;
    return SPREG_OK;
}

int execute_batched_impl(const spreg_work_item *items, int32_t n, cudaStream_t stream) {
    SPREG_CHECK_ARG(n >= 0 && (n == 0 || items), "bad work list");
    std::vector<const spreg_packed *> as((size_t)n);
    std::vector<const spreg_exec_args *> args((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        as[i] = items[i].a;
        args[i] = &items[i].args;
    }
    return run_calls(as.data(), args.data(), n, stream);
}

}  // namespace spreg
