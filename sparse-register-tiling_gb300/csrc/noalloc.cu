// noalloc.cu -- spreg_execute_batched_noalloc: the batched SpMM executor for callers that cannot
// allocate device memory when they run it.
//
// Who needs it: code that executes pruned layers inside a region where it must not call
// cudaMalloc -- a serving loop whose device memory is owned by another allocator (a framework's
// caching allocator, a fixed arena sized at start-up), code that must not add the implicit device
// synchronisation a first-time cudaMalloc can cause, or a real-time path that promises no
// allocation after warm-up.  The regular entry point (spreg_execute_batched) allocates a small
// per-device pool on its first call; this one never does.
//
// The only scratch the batched kernel needs is one work counter per launch and a status word.
// Here they live in g_noalloc_scratch, a file-scope device array that every GPU loading the
// library holds until the process exits: slot 0 is the status word, slots 1 .. 64 the counters,
// so one call may issue at most kNoAllocLaunches launches (one per group of at most 224 SpMMs of
// one configuration).  Larger calls are rejected.  Host code cannot use the array's name as a
// device address (it is a host-side stand-in), so the first call on each device looks the address
// up with cudaGetSymbolAddress while that device is current; make that first call before any
// stream capture.  Every call shares the array and clears the counters it uses before its
// launches, so calls whose work overlaps on the GPU (other streams, other threads) race on it.  The
// status word keeps its value until spreg_device_status reads and clears it (that call reports the
// word of the regular executors and this one's).
#include "exec_kernel.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace spreg {

int auto_nv(int64_t n, int64_t panels, int sms, int64_t others1);  // exec.cu
int64_t strip_items1(const spreg_packed *a, const spreg_exec_args *args);  // exec.cu

constexpr int kNoAllocLaunches = 64;
static __device__ __align__(256) int g_noalloc_scratch[1 + kNoAllocLaunches];

namespace {

struct NoAllocDevice {
    int *scratch = nullptr;  // device address of g_noalloc_scratch
    int sms = 0, smem_optin = 0, smem_per_sm = 0;
};

std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[64];

// Set-up, once per device, with that device current: the scratch address and launch limits.
int noalloc_device(NoAllocDevice **out) {
    int dev = 0;
    SPREG_CUDA(cudaGetDevice(&dev));
    SPREG_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.scratch) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            SPREG_FAIL(SPREG_ERR_CUDA, "cudaGetSymbolAddress(no-allocation scratch) failed: %s", cudaGetErrorString(e));
        SPREG_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
        SPREG_CUDA(cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        SPREG_CUDA(cudaDeviceGetAttribute(&d.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        if (d.smem_optin > kMaxSmem) d.smem_optin = kMaxSmem;
        d.scratch = static_cast<int *>(ptr);
    }
    *out = &d;
    return SPREG_OK;
}

int combo_code(int vt, int bt, int ct) {
    if (vt == SPREG_F32 && bt == SPREG_F32 && ct == SPREG_F32) return COMBO_F32;
    if (vt == SPREG_BF16 && bt == SPREG_BF16 && ct == SPREG_F32) return COMBO_BF16_F32OUT;
    if (vt == SPREG_BF16 && bt == SPREG_BF16 && ct == SPREG_BF16) return COMBO_BF16_BF16OUT;
    if (vt == SPREG_F16 && bt == SPREG_F16 && ct == SPREG_F32) return COMBO_F16_F32OUT;
    return -1;
}

template <int MR>
cudaError_t noalloc_launch_combo(const BatchParams &p, int nv, int combo, unsigned grid, int threads, size_t smem,
                                 cudaStream_t s) {
    switch (combo) {
    case COMBO_F32: return launch_exec_batch<MR, COMBO_F32>(p, nv, grid, threads, smem, s);
    case COMBO_BF16_F32OUT: return launch_exec_batch<MR, COMBO_BF16_F32OUT>(p, nv, grid, threads, smem, s);
    case COMBO_BF16_BF16OUT: return launch_exec_batch<MR, COMBO_BF16_BF16OUT>(p, nv, grid, threads, smem, s);
    case COMBO_F16_F32OUT: return launch_exec_batch<MR, COMBO_F16_F32OUT>(p, nv, grid, threads, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t noalloc_launch(int mr, const BatchParams &p, int nv, int combo, unsigned grid, int threads, size_t smem,
                           cudaStream_t s) {
    switch (mr) {
    case 2: return noalloc_launch_combo<2>(p, nv, combo, grid, threads, smem, s);
    case 4: return noalloc_launch_combo<4>(p, nv, combo, grid, threads, smem, s);
    case 6: return noalloc_launch_combo<6>(p, nv, combo, grid, threads, smem, s);
    case 8: return noalloc_launch_combo<8>(p, nv, combo, grid, threads, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

struct NoAllocGroup {
    int mr = 0, combo = 0, nv = 0;
    int64_t xbuf = 0;
    std::vector<XProblem> probs;
};

bool is_aligned(const void *p, size_t bytes) { return (reinterpret_cast<uintptr_t>(p) % bytes) == 0; }

}  // namespace

// Status word of the no-allocation entry point on device `dev` (*have = false if that entry point
// was never set up there): read, and cleared when reset != 0.  For spreg_device_status.
int noalloc_status_word(int dev, int32_t *v, int reset, bool *have) {
    *have = false;
    *v = 0;
    if (dev < 0 || dev >= 64) return SPREG_OK;
    int *w = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        w = g_noalloc_dev[dev].scratch;
    }
    if (!w) return SPREG_OK;
    *have = true;
    SPREG_CUDA(cudaMemcpy(v, w, sizeof(int), cudaMemcpyDeviceToHost));
    if (reset) SPREG_CUDA(cudaMemset(w, 0, sizeof(int)));
    return SPREG_OK;
}

}  // namespace spreg

using namespace spreg;

extern "C" int spreg_execute_batched_noalloc(const spreg_work_item *items, int32_t num_items, spreg_stream_t stream) {
    clear_error();
    SPREG_CHECK_ARG(num_items >= 0 && (num_items == 0 || items), "bad work list");
    NoAllocDevice *d;
    int st = noalloc_device(&d);
    if (st != SPREG_OK) return st;
    int dev = -1;
    SPREG_CUDA(cudaGetDevice(&dev));
    cudaStream_t s = (cudaStream_t)stream;

    // Plan every SpMM as the batched kernel's problems (whole strips + an NV = 1 remainder).
    std::map<std::tuple<int, int, int>, NoAllocGroup> groups;
    int64_t items1 = 0;
    for (int32_t i = 0; i < num_items; ++i) items1 += strip_items1(items[i].a, &items[i].args);
    for (int32_t i = 0; i < num_items; ++i) {
        const spreg_packed *a = items[i].a;
        const spreg_exec_args *args = &items[i].args;
        SPREG_CHECK_ARG(a, "work item %d has no packed matrix", i);
        const spreg_packed_info &in = a->info;
        SPREG_CHECK_ARG(a->device == dev, "work item %d: packed matrix lives on device %d, current device is %d", i,
                        a->device, dev);
        const int combo = combo_code(in.value_dtype, args->b_dtype, args->c_dtype);
        SPREG_CHECK_ARG(combo >= 0, "work item %d: unsupported dtype combination", i);
        SPREG_CHECK_ARG(args->n >= 0 && args->ldc >= args->n && (args->ldb >= args->n || in.cols == 0),
                        "work item %d: bad n / ldb / ldc", i);
        SPREG_CHECK_ARG(args->n == 0 || in.rows == 0 || (args->c && (args->b || in.cols == 0)),
                        "work item %d: null B or C", i);
        SPREG_CHECK_ARG(args->epilogue == SPREG_EPILOGUE_NONE || args->epilogue == SPREG_EPILOGUE_RELU,
                        "work item %d: bad epilogue", i);
        SPREG_CHECK_ARG(args->job_order == 0 || args->job_order == 1, "work item %d: job_order must be 0 or 1", i);
        SPREG_CHECK_ARG(args->b_staging != 1 && args->meta_staging != 2 && args->panel_rounds <= 1 &&
                            args->load_balance == 0,
                        "work item %d: the no-allocation entry point runs the batched execution-layout kernel only", i);
        const int64_t xbuf = (a->max_exec_bytes + 127) / 128 * 128;
        SPREG_CHECK_ARG(a->exec && 1024 + 2 * xbuf <= d->smem_optin,
                        "work item %d: execution blocks (%lld bytes) too large for the batched kernel", i,
                        (long long)a->max_exec_bytes);
        int nv;
        switch (args->nr) {
        case 0: nv = auto_nv(args->n, in.num_panels, d->sms, items1 - strip_items1(a, args)); break;
        case 32: nv = 1; break;
        case 64: nv = 2; break;
        case 128: nv = 4; break;
        case 256: nv = 4; break;  // wide strips below where the gather kernel has them, else 128
        case 512: nv = 4; break;
        default: SPREG_FAIL(SPREG_ERR_INVALID_ARG, "work item %d: nr must be 0, 32, 64, 128, 256 or 512", i);
        }
        const size_t bsz = dtype_bytes(args->b_dtype), csz = dtype_bytes(args->c_dtype);
        while (nv > 1 && !(is_aligned(args->b, bsz * nv) && args->ldb % nv == 0 && is_aligned(args->c, csz * nv) &&
                           args->ldc % nv == 0))
            nv >>= 1;
        // the gather kernel's wide strips, as spreg_execute chooses them: FP32 256 columns (512 at
        // M_r <= 4), 16-bit B 256 and 512 columns at M_r <= 4
        if ((args->nr == 256 || args->nr == 512) && nv == 4 && args->n >= 256 && is_aligned(args->b, 16) &&
            is_aligned(args->c, 16)) {
            const bool wide32 = combo == COMBO_F32 && args->ldb % 4 == 0 && args->ldc % 4 == 0;
            const bool wide16 = bsz == 2 && in.mr <= 4 && args->ldb % 8 == 0 && is_aligned(args->c, csz * 8) &&
                                args->ldc % 8 == 0;
            const bool w512 = args->nr == 512 && in.mr <= 4 && args->n >= 512;
            if (wide32 || wide16) nv = w512 ? 16 : 8;
        }
        const int64_t n_main = (args->n / (32 * nv)) * (32 * nv);
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
        if (base.P == 0) continue;
        auto add = [&](int64_t c0, int64_t c1, int32_t strips, int v) {
            XProblem pr = base;
            pr.col_begin = c0;
            pr.col_end = c1;
            pr.S = strips;
            NoAllocGroup &g = groups[std::make_tuple(in.mr, combo, v)];
            g.mr = in.mr;
            g.combo = combo;
            g.nv = v;
            g.xbuf = std::max(g.xbuf, xbuf);
            g.probs.push_back(pr);
        };
        if (n_main > 0) add(0, n_main, (int32_t)(n_main / (32 * nv)), nv);
        if (args->n > n_main) add(n_main, args->n, (int32_t)((args->n - n_main + 31) / 32), 1);
    }
    int64_t launches = 0;
    for (auto &kv : groups) launches += ((int64_t)kv.second.probs.size() + kMaxBatchProblems - 1) / kMaxBatchProblems;
    SPREG_CHECK_ARG(launches <= kNoAllocLaunches,
                    "this work list needs %lld launches; the no-allocation entry point has scratch for at most %d "
                    "(each launch runs up to %d SpMMs of one M_r / strip width / dtype combination)",
                    (long long)launches, kNoAllocLaunches, kMaxBatchProblems);

    // Clear every counter this call uses, then launch.  The status word keeps what earlier calls
    // recorded until spreg_device_status reads and clears it.
    int *scratch = d->scratch;
    if (launches > 0) SPREG_CUDA(cudaMemsetAsync(scratch + 1, 0, sizeof(int) * (size_t)launches, s));
    int slot = 0;
    for (auto &kv : groups) {
        NoAllocGroup &g = kv.second;
        for (size_t first = 0; first < g.probs.size(); first += kMaxBatchProblems) {
            const size_t cnt = std::min<size_t>(kMaxBatchProblems, g.probs.size() - first);
            BatchParams bp;
            bp.nprob = (int32_t)cnt;
            int64_t total = 0;
            for (size_t i = 0; i < cnt; ++i) {
                bp.prob[i] = g.probs[first + i];
                bp.prob[i].item_begin = total;
                total += (int64_t)bp.prob[i].P * bp.prob[i].S;
            }
            ++slot;
            if (total == 0) continue;
            SPREG_CHECK_ARG(total <= INT32_MAX, "too many work items in one launch");
            bp.items = total;
            bp.xbuf = (int32_t)g.xbuf;
            bp.status = scratch;
            bp.counter = scratch + slot;
            int nw = g.nv >= 8 && g.combo == COMBO_F32 ? kWideMaxWarps : 8;  // wide FP32: the kernel's bound
            while (nw > 1 && 1024 + 2 * g.xbuf * nw > d->smem_optin) nw >>= 1;
            const size_t smem = (size_t)(1024 + 2 * g.xbuf * nw);
            const int threads = 32 * nw;
            const int per_sm = std::max(1, std::min((int)(d->smem_per_sm / (int64_t)smem), 2048 / threads));
            const int64_t ctas = std::min<int64_t>((int64_t)d->sms * per_sm, (total + nw - 1) / nw);
            cudaError_t e = noalloc_launch(g.mr, bp, g.nv, g.combo, (unsigned)ctas, threads, smem, s);
            if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "batched executor launch: %s", cudaGetErrorString(e));
        }
    }
    return SPREG_OK;
}
