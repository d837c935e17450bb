// exec.cu -- host side of the executor: argument checks, strip-width choice, launches.
#include "exec_kernel.cuh"

#include <algorithm>
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

}  // namespace

// Floats per lane chosen automatically: wide strips amortise the per-entry index and value
// loads over more columns, narrow strips give more warps when N is small.
int auto_nv(int64_t n, int64_t panels) {
    int nv = 1;
    if (n >= 64) nv = 2;
    if (n >= 128) nv = 4;
    // keep at least ~4 warps per SM of work
    while (nv > 1 && panels * ((n + 32 * nv - 1) / (32 * nv)) < 152 * 4) nv >>= 1;
    return nv;
}

struct LaunchPlan {
    ExecParams p;
    int mr, combo, nv, warps;
    int64_t n_main;  // columns covered by the NV launch (whole strips)
};

int plan_exec(const spreg_packed *a, const spreg_exec_args *args, LaunchPlan *lp) {
    SPREG_CHECK_ARG(a && args, "null packed matrix or args");
    const spreg_packed_info &in = a->info;
    const int combo = combo_of(in.value_dtype, args->b_dtype, args->c_dtype);
    SPREG_CHECK_ARG(combo >= 0, "unsupported dtype combination values=%d B=%d C=%d (B must match the values; "
                    "C is F32, or BF16 for BF16 values)", in.value_dtype, args->b_dtype, args->c_dtype);
    SPREG_CHECK_ARG(args->n >= 0, "n must be >= 0");
    SPREG_CHECK_ARG(args->n == 0 || in.rows == 0 || (args->c && (args->b || in.cols == 0)), "null B or C");
    SPREG_CHECK_ARG(args->ldb >= args->n || in.cols == 0, "ldb (%lld) < n (%lld)", (long long)args->ldb, (long long)args->n);
    SPREG_CHECK_ARG(args->ldc >= args->n, "ldc (%lld) < n (%lld)", (long long)args->ldc, (long long)args->n);
    SPREG_CHECK_ARG(args->epilogue == SPREG_EPILOGUE_NONE || args->epilogue == SPREG_EPILOGUE_RELU, "bad epilogue");
    int nv;
    switch (args->nr) {
    case 0: nv = auto_nv(args->n, in.num_panels); break;
    case 32: nv = 1; break;
    case 64: nv = 2; break;
    case 128: nv = 4; break;
    case 256: nv = 8; break;
    default: SPREG_FAIL(SPREG_ERR_INVALID_ARG, "nr must be 0, 32, 64, 128 or 256 (got %d)", args->nr);
    }
    const size_t bsz = dtype_bytes(args->b_dtype), csz = dtype_bytes(args->c_dtype);
    while (nv > 1 && !(aligned(args->b, bsz * nv) && args->ldb % nv == 0 && aligned(args->c, csz * nv) &&
                       args->ldc % nv == 0))
        nv >>= 1;
    int warps = args->warps_per_cta > 0 ? args->warps_per_cta : 4;
    SPREG_CHECK_ARG(warps >= 1 && warps <= 8, "warps_per_cta must be in [1, 8]");

    ExecParams &p = lp->p;
    p.arena = a->arena;
    p.descs = a->descs;
    p.scales = a->scales;
    p.B = args->b;
    p.C = args->c;
    p.ldb = args->ldb;
    p.ldc = args->ldc;
    p.M = in.rows;
    p.N = args->n;
    p.col_begin = 0;
    p.P = a->geom.P;
    p.ppt = a->geom.ppt;
    p.T = a->geom.T;
    p.nk = in.num_nkern;
    p.load_c = args->load_c ? 1 : 0;
    p.epilogue = args->epilogue;
    p.pad_ = 0;
    for (int i = 0; i < 256; ++i) p.id_pattern[i] = a->id_to_pattern[i];
    lp->mr = in.mr;
    lp->combo = combo;
    lp->nv = nv;
    lp->warps = warps;
    lp->n_main = nv > 1 ? (args->n / (32 * nv)) * (32 * nv) : 0;
    return SPREG_OK;
}

int launch_plan(const LaunchPlan &lp, cudaStream_t stream) {
    if (lp.p.N == 0 || lp.p.P == 0) return SPREG_OK;
    const unsigned gx = (unsigned)((lp.p.P + lp.warps - 1) / lp.warps);
    const int threads = 32 * lp.warps;
    SPREG_CHECK_ARG(gx <= 0x7FFFFFFFu, "too many panels");
    if (lp.n_main > 0) {
        const int64_t gy = lp.n_main / (32 * lp.nv);
        SPREG_CHECK_ARG(gy <= 65535, "n too large for one launch");
        ExecParams p = lp.p;
        p.col_begin = 0;
        cudaError_t e = launch_mr(lp.mr, p, lp.nv, lp.combo, dim3(gx, (unsigned)gy), threads, stream);
        if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "executor launch: %s", cudaGetErrorString(e));
    }
    const int64_t tail = lp.p.N - lp.n_main;
    if (tail > 0) {
        const int64_t gy = (tail + 31) / 32;
        SPREG_CHECK_ARG(gy <= 65535, "n too large for one launch");
        ExecParams p = lp.p;
        p.col_begin = lp.n_main;
        cudaError_t e = launch_mr(lp.mr, p, 1, lp.combo, dim3(gx, (unsigned)gy), threads, stream);
        if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "executor launch: %s", cudaGetErrorString(e));
    }
    return SPREG_OK;
}

int execute_impl(const spreg_packed *a, const spreg_exec_args *args, cudaStream_t stream) {
    LaunchPlan lp;
    int st = plan_exec(a, args, &lp);
    if (st != SPREG_OK) return st;
    int dev = -1;
    SPREG_CUDA(cudaGetDevice(&dev));
    SPREG_CHECK_ARG(dev == a->device, "packed matrix lives on device %d, current device is %d", a->device, dev);
    return launch_plan(lp, stream);
}

int execute_timed_impl(const spreg_packed *a, const spreg_exec_args *args, int64_t num_runs, double *median_ns,
                       cudaStream_t stream) {
    SPREG_CHECK_ARG(median_ns, "null median_ns");
    SPREG_CHECK_ARG(num_runs >= 1, "num_runs must be >= 1");
    LaunchPlan lp;
    int st = plan_exec(a, args, &lp);
    if (st != SPREG_OK) return st;
    const int kIters = 150;  // MEASURED_ITERATIONS of template:317
    for (int64_t r = 0; r < num_runs; ++r)
        if ((st = launch_plan(lp, stream))) return st;
    std::vector<cudaEvent_t> ev(2 * kIters);
    for (auto &e : ev) SPREG_CUDA(cudaEventCreate(&e));
    for (int it = 0; it < kIters; ++it) {
        cudaEventRecord(ev[2 * it], stream);
        for (int64_t r = 0; r < num_runs; ++r)
            if ((st = launch_plan(lp, stream))) break;
        cudaEventRecord(ev[2 * it + 1], stream);
        if (st) break;
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
    std::vector<LaunchPlan> plans((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        int st = plan_exec(items[i].a, &items[i].args, &plans[i]);
        if (st != SPREG_OK) return st;
    }
    for (int32_t i = 0; i < n; ++i) {
        int st = launch_plan(plans[i], stream);
        if (st != SPREG_OK) return st;
    }
    return SPREG_OK;
}

}  // namespace spreg
