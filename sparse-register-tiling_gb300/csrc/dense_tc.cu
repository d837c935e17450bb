// dense_tc.cu -- dense row panels on the 5th-generation tensor cores (tcgen05 MMA, tensor memory,
// TMA).
//
// C[row_index[i], 0:n] (+)= A_rows[i, 0:K] . B[0:K, 0:n] for the rows of a pruned matrix whose panels
// are dense enough that a tensor-core product beats the register-tiled executors.  Two operand forms:
//   * BF16 (spreg_dense_rows_bf16): BF16 A and B, FP32 accumulation in tensor memory (TMEM), FP32 or
//     BF16 output;
//   * FP32-accurate split (spreg_dense_rows_f32): FP32 A and B, each scaled by a power of two (A per
//     row, B per column) and split into two FP16 halves, x = hi + lo with hi = fp16(x) and
//     lo = fp16(x - hi).  Three FP16 MMAs per K step, hi.hi + hi.lo + lo.hi, accumulate in FP32;
//     the dropped lo.lo term and the rounding of lo are below 2^-22 of each product, the level of
//     FP32's own rounding.  The epilogue undoes the scales (exact powers of two).  The tensor core
//     accumulates in FP32 with truncation, an error that grows with the 16-deep K steps of one
//     accumulator, so K is cut into chunks of TC_SPLIT_CHUNK run by successive launches that add
//     into C.
// load_c and the ReLU epilogue apply to both.
//
// One launch runs up to TC_MAX_PROBLEMS products ("problems"; their tensor maps sit in a device
// table).  Its output tiles (128 rows x BN columns; BN 256 when every product of the launch has
// more than 128 columns, else 128) are shared out over persistent CTAs of 10 warps, at most one per
// SM, each finding a tile's problem by a binary search over the problems' first tiles:
//   * warp 0 (one lane) loads 64-deep K blocks of A_rows (128 x 64, K-major) and of B into a ring of
//     stages with 2-D tensor copies (TMA, 128-byte swizzle; "full" mbarriers with expected bytes).
//     A single BF16 product's B, and every split product's B halves, are read as N-major operands
//     (BN / 64 copies of 64 columns x 64 K rows); BF16 products coalesced over several B are first
//     transposed into one K-major buffer;
//   * warp 1 (one lane) issues tcgen05.mma.kind::f16 (M 128, N BN, K 16; four per K block, twelve for
//     a split product) into one of two TMEM accumulators, tcgen05.commit releasing the stage
//     ("empty") and, per tile, the accumulator ("acc full");
//   * warps 2-9 each read one 32-lane quarter of the accumulator (the tile's rows) and half of its
//     columns with tcgen05.ld, apply the scales, load_c and ReLU, store through the row index (and
//     the segment table of coalesced products) and release the accumulator ("acc empty"), so the
//     next tile's MMAs overlap these stores.
// Columns past n are zero-filled by the tensor copies and never stored; K past the end of A reads
// as zero; rows past R are never stored.  Every wait is bounded: a wait that gives up records a
// code in the device status word; TMEM is released on every path.
#include "spreg_common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

namespace spreg {

int *device_status_word(int *st);  // exec.cu

namespace {

constexpr int TC_BM = 128, TC_BK = 64;
// K block of a split product: 64 deep (128-byte rows, 128-byte swizzle) as for BF16, its four operand
// tiles (A hi, A lo, B hi, B lo) making stages of 96 KB (two in flight) for 256-wide tiles and 64 KB
// (three) for 128-wide ones.  Measured against 32-deep blocks with the 64-byte swizzle and four
// stages of 48 KB: 11-25 % faster (half the tensor copies per byte, 128-byte rows).
constexpr int TC_BK_SPLIT = 64;
template <bool SPLIT> constexpr int tc_bk() { return SPLIT ? TC_BK_SPLIT : TC_BK; }
// Output tile width BN (128 or 256): the MMA's N, the TMEM accumulator's columns, B tile rows.
// A split product stages both halves of A and of B.
template <int BN, bool SPLIT> constexpr uint32_t tc_tile_a() { return (uint32_t)TC_BM * tc_bk<SPLIT>() * 2; }
template <int BN, bool SPLIT = false> constexpr uint32_t tc_tile_b() { return (uint32_t)BN * tc_bk<SPLIT>() * 2; }
template <int BN, bool SPLIT> constexpr uint32_t tc_stage() {
    return (SPLIT ? 2u : 1u) * (tc_tile_a<BN, SPLIT>() + tc_tile_b<BN, SPLIT>());
}
// Stages of the ring: about 190 KB of operands.
template <int BN, bool SPLIT> constexpr int tc_stages() { return !SPLIT ? 4 : BN == 256 ? 2 : 3; }
// Epilogue warps: two per TMEM lane quarter, each storing half of the tile's columns.
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_THREADS = 32 * (2 + TC_EPI_WARPS);
// The epilogue warps' staging buffers: 8 x 32 rows x 33 floats.
constexpr uint32_t TC_EPI_BYTES = (uint32_t)TC_EPI_WARPS * 32u * 33u * 4u;
template <int BN, bool SPLIT> constexpr size_t tc_smem() {
    return 1024 /* alignment slack */ + tc_stages<BN, SPLIT>() * tc_stage<BN, SPLIT>() + 256 /* barriers, TMEM slot */ +
           TC_EPI_BYTES;
}

static_assert(tc_smem<256, true>() <= 232448 && tc_smem<128, true>() <= 232448 && tc_smem<256, false>() <= 232448 &&
                  tc_smem<128, false>() <= 232448,
              "tensor-core kernel shared memory exceeds 227 KB per CTA");

constexpr int TC_MAX_PROBLEMS = 192;  // problems per launch (kernel parameters <= 32 KB)
// K per pass of a split product (a multiple of TC_BK): bounds the MMA steps of one accumulator.
constexpr int64_t TC_SPLIT_CHUNK = 1024;

struct TcProblem {
    // Tensor maps in the launch's device table (64-byte aligned):
    const CUtensorMap *a_map;  // A_rows: columns [0, K) x rows, box 64 x 128, 128-byte swizzle
    const CUtensorMap *b_map;  // Bt: columns [0, K) x rows [0, n), box 64 x BN; or (b_mn) B itself:
                               // columns [0, n) x rows, box 64 x 64
    const int32_t *row_index;  // output row of each A row
    void *C;
    int64_t ldc;
    int32_t R, n, kblocks, c_dtype;
    int32_t load_c, epilogue, tile_begin, tiles_n;  // first output tile of the launch, tiles along n
    // Products sharing A (same weight rows, row index and epilogue) are one problem whose columns
    // are their B's side by side: column j belongs to segment s with seg_start[s] <= j <
    // seg_start[s + 1] and is column j - seg_start[s] of C seg_c[s] (row stride seg_ldc[s]).
    const int32_t *seg_start;
    void *const *seg_c;
    const int64_t *seg_ldc;
    int32_t nseg;
    int32_t b_mn;              // B read as an N-major operand, no transpose
    // Split products: A's low halves are rows [a_lo_row, a_lo_row + R) of the A map, B's rows
    // [b_lo_row, 2 b_lo_row) of the B map; C = acc * row_scale[r] * col_scale[j].
    int32_t a_lo_row, b_lo_row;
    const float *row_scale, *col_scale;
    // First K block of this problem: a long split product runs as K chunks, one per launch, each
    // accumulating into C (the tensor core's FP32 accumulation truncates, so its error grows with
    // the K steps of one accumulator; a chunk bounds them).
    int32_t kb0, pad1;
};

struct TcParams {
    int *status;
    int32_t nprob, pad0;
    TcProblem prob[TC_MAX_PROBLEMS];
};
static_assert(sizeof(TcParams) <= 32764, "kernel parameters are limited to 32764 bytes");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tc_mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool tc_try_wait(uint32_t bar, uint32_t phase) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t phase, int *status, int code) {
    for (uint32_t it = 0; it < (1u << 22); ++it)
        if (tc_try_wait(bar, phase)) return true;
    if (status) atomicCAS(status, 0, code);
    return false;
}
__device__ __forceinline__ void mbar_arrive_tc(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Tensor maps live in global memory, written by a host copy before the launch: make them visible
// to the tensor-map proxy before the first copy through them.
__device__ __forceinline__ void tc_map_acquire(const CUtensorMap *map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}
__device__ __forceinline__ void tc_tma_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile stored with the 128-byte swizzle: rows of
// 128 bytes (64 BF16), 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address, 16-byte units
    d |= (uint64_t)1 << 16;                    // leading-dimension byte offset (unused for this layout)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride-dimension byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                    // descriptor version of tcgen05
    d |= (uint64_t)2 << 61;                    // layout: 128-byte swizzle
    return d;
}

// Shared-memory matrix descriptor of an N-major (MN-major) operand tile with the 128-byte swizzle:
// each K row holds 64 BF16 of N in 128 bytes, 8-row K groups are 1024 bytes apart (stride), and
// 64-column N blocks (one tensor copy of 64 K rows each) are 8192 bytes apart (leading dimension).
__device__ __forceinline__ uint64_t tc_desc_mn(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address, 16-byte units
    d |= (uint64_t)(8192 >> 4) << 16;          // leading-dimension byte offset: next 64-column N block
    d |= (uint64_t)(1024 >> 4) << 32;          // stride-dimension byte offset: next 8-row K group
    d |= (uint64_t)1 << 46;                    // descriptor version of tcgen05
    d |= (uint64_t)2 << 61;                    // layout: 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16 (bf16) or FP16, both K-major, M x N.
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N, bool bf16 = true) {
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive accumulator columns of the warp's 32 TMEM lanes, issued without waiting;
// tc_ld32_wait completes it.  The wait takes the same registers as operands, so no use of them can be
// scheduled above it.
__device__ __forceinline__ void tc_ld32_issue(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
}
__device__ __forceinline__ void tc_ld32_wait(uint32_t (&r)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory");
}

// Problem of output tile t of the launch (binary search over the problems' first tiles).
__device__ __forceinline__ int tc_problem_of(const TcParams &p, int t) {
    int lo = 0, hi = p.nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p.prob[mid].tile_begin <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Epilogue constants of one output tile, read once from the problem (kernel parameter space).
struct TcEpi {
    void *C;
    int64_t ldc;
    int n, c_dtype, load_c, epilogue, nseg;
    const int32_t *seg_start;
    void *const *seg_c;
    const int64_t *seg_ldc;
    const float *col_scale;
};
__device__ __forceinline__ TcEpi tc_epi_of(const TcProblem &q) {
    TcEpi e;
    e.C = q.C;
    e.ldc = q.ldc;
    e.n = q.n;
    e.c_dtype = q.c_dtype;
    e.load_c = q.load_c;
    e.epilogue = q.epilogue;
    e.nseg = q.nseg;
    e.seg_start = q.seg_start;
    e.seg_c = q.seg_c;
    e.seg_ldc = q.seg_ldc;
    e.col_scale = q.col_scale;
    return e;
}

// One 32-column chunk of the epilogue (columns n0 + c .. + 31, registers r from TMEM, lane i holding
// tile row i): scales (split products: (acc * row_scale) * col_scale, each factor a power of two),
// load_c / ReLU, store.
//
// Whole 32-column chunks of one output go through the warp's 32 x 33 shared-memory buffer `eb`:
// lane i writes row i's 32 raw values, then each store instruction covers 4 rows x 32 columns (8
// lanes x 16 bytes per row), where a lane storing its own row would scatter 32 rows per
// instruction.  The 33-float row pitch keeps both passes free of bank conflicts.  The scales are
// applied after the transpose (a lane's 4 columns keep their 4 column scales for the whole chunk);
// with load_c the chunk's 8 reads of C are issued before any of them is used.
template <bool SPLIT>
__device__ __forceinline__ void tc_store_chunk(const TcEpi &e, int n0, int c, int lane, const uint32_t (&r)[32],
                                               float rs, bool row_ok, long long orow, bool vec_ok, int &seg,
                                               float *eb) {
    if (n0 + c >= e.n) return;  // uniform: a chunk past the last column
    // output of this chunk: C itself, or (coalesced products) the segment it lies in, when it lies in one
    void *cbase = e.C;
    int64_t cld = e.ldc;
    int ccol = n0 + c;
    bool whole = vec_ok && n0 + c + 32 <= e.n;
    if (e.nseg > 1) {
        while (n0 + c >= e.seg_start[seg + 1]) ++seg;  // uniform: every lane sees the same columns
        const int esz = e.c_dtype == SPREG_F32 ? 4 : 2;
        cbase = e.seg_c[seg];
        cld = e.seg_ldc[seg];
        ccol = n0 + c - e.seg_start[seg];
        whole = n0 + c + 32 <= e.seg_start[seg + 1] && (reinterpret_cast<uintptr_t>(cbase) % (4 * esz)) == 0 &&
                (cld % 4) == 0 && (ccol % 4) == 0;
    }
    if (whole) {  // uniform over the warp
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 32; ++j) eb[lane * 33 + j] = __uint_as_float(r[j]);
        const int c4 = (lane & 7) * 4;
        float cs[4] = {1.0f, 1.0f, 1.0f, 1.0f};
        if constexpr (SPLIT) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(e.col_scale + n0 + c + c4));
            cs[0] = v.x; cs[1] = v.y; cs[2] = v.z; cs[3] = v.w;
        }
        // rows of this lane's 8 stores: 4 * it + lane / 8
        long long orow_r[8];
        bool ok_r[8];
        float rs_r[8];
#pragma unroll
        for (int it = 0; it < 8; ++it) {
            const int rr = 4 * it + (lane >> 3);
            ok_r[it] = __shfl_sync(0xffffffffu, row_ok, rr);
            orow_r[it] = __shfl_sync(0xffffffffu, orow, rr);
            rs_r[it] = SPLIT ? __shfl_sync(0xffffffffu, rs, rr) : 1.0f;
        }
        __syncwarp();
        if (e.c_dtype == SPREG_F32) {
            float4 *cp[8];
            float4 ci[8];
#pragma unroll
            for (int it = 0; it < 8; ++it) {
                cp[it] = reinterpret_cast<float4 *>(reinterpret_cast<float *>(cbase) + orow_r[it] * cld + ccol + c4);
                ci[it] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (e.load_c && ok_r[it]) ci[it] = *cp[it];
            }
#pragma unroll
            for (int it = 0; it < 8; ++it) {
                const int rr = 4 * it + (lane >> 3);
                float o[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    o[t] = eb[rr * 33 + c4 + t];
                    if constexpr (SPLIT) o[t] = (o[t] * rs_r[it]) * cs[t];
                }
                if (e.load_c) {
                    o[0] += ci[it].x; o[1] += ci[it].y; o[2] += ci[it].z; o[3] += ci[it].w;
                }
                if (e.epilogue == SPREG_EPILOGUE_RELU)
#pragma unroll
                    for (int t = 0; t < 4; ++t) o[t] = fmaxf(o[t], 0.0f);
                if (ok_r[it]) *cp[it] = make_float4(o[0], o[1], o[2], o[3]);
            }
        } else {
            uint2 *cp[8];
            uint2 ci[8];
#pragma unroll
            for (int it = 0; it < 8; ++it) {
                cp[it] = reinterpret_cast<uint2 *>(reinterpret_cast<__nv_bfloat16 *>(cbase) + orow_r[it] * cld + ccol + c4);
                ci[it] = make_uint2(0u, 0u);
                if (e.load_c && ok_r[it]) ci[it] = *cp[it];
            }
#pragma unroll
            for (int it = 0; it < 8; ++it) {
                const int rr = 4 * it + (lane >> 3);
                float o[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    o[t] = eb[rr * 33 + c4 + t];
                    if constexpr (SPLIT) o[t] = (o[t] * rs_r[it]) * cs[t];
                }
                if (e.load_c) {
                    const __nv_bfloat162 c01 = *reinterpret_cast<const __nv_bfloat162 *>(&ci[it].x);
                    const __nv_bfloat162 c23 = *reinterpret_cast<const __nv_bfloat162 *>(&ci[it].y);
                    o[0] += __low2float(c01); o[1] += __high2float(c01);
                    o[2] += __low2float(c23); o[3] += __high2float(c23);
                }
                if (e.epilogue == SPREG_EPILOGUE_RELU)
#pragma unroll
                    for (int t = 0; t < 4; ++t) o[t] = fmaxf(o[t], 0.0f);
                __nv_bfloat162 w01 = __floats2bfloat162_rn(o[0], o[1]), w23 = __floats2bfloat162_rn(o[2], o[3]);
                uint2 w;
                w.x = *reinterpret_cast<uint32_t *>(&w01);
                w.y = *reinterpret_cast<uint32_t *>(&w23);
                if (ok_r[it]) *cp[it] = w;
            }
        }
        return;
    }
    if (!row_ok) return;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int col = n0 + c + j;
        if (col >= e.n) break;
        void *cb = e.C;
        int64_t ldc = e.ldc;
        int lcol = col;
        if (e.nseg > 1) {
            while (col >= e.seg_start[seg + 1]) ++seg;
            cb = e.seg_c[seg];
            ldc = e.seg_ldc[seg];
            lcol = col - e.seg_start[seg];
        }
        float o = __uint_as_float(r[j]);
        if constexpr (SPLIT) o = (o * rs) * __ldg(e.col_scale + col);
        if (e.c_dtype == SPREG_F32) {
            float *cp = reinterpret_cast<float *>(cb) + orow * ldc + lcol;
            if (e.load_c) o += *cp;
            if (e.epilogue == SPREG_EPILOGUE_RELU) o = fmaxf(o, 0.0f);
            *cp = o;
        } else {
            __nv_bfloat16 *cp = reinterpret_cast<__nv_bfloat16 *>(cb) + orow * ldc + lcol;
            if (e.load_c) o += __bfloat162float(*cp);
            if (e.epilogue == SPREG_EPILOGUE_RELU) o = fmaxf(o, 0.0f);
            *cp = __float2bfloat16_rn(o);
        }
    }
}

// Row index and (split) row scale of lane `lane`'s tile row, read before the accumulator is ready.
struct TcRowInfo {
    long long orow;
    float rs;
    bool ok;
};
template <bool SPLIT>
__device__ __forceinline__ TcRowInfo tc_row_info(const TcProblem &q, int m0, int quarter, int lane) {
    const int r = m0 + 32 * quarter + lane;
    TcRowInfo ri;
    ri.ok = r < q.R;
    ri.orow = ri.ok ? q.row_index[r] : 0;
    ri.rs = (SPLIT && ri.ok) ? q.row_scale[r] : 1.0f;
    return ri;
}

// Epilogue of one output tile by one warp: TMEM lanes 32 * quarter .. + 31 (tile rows) and columns
// [c0, c0 + NC) of the accumulator at TMEM address tacc (lane 0, its first column); store through
// the row index (and segments).  The TMEM load of chunk c + 1 is issued before chunk c is
// processed, so the TMEM latency overlaps the stores.
template <int NC, bool SPLIT>
__device__ __forceinline__ void tc_store_tile(const TcEpi &e, int n0, int c0, int quarter, int lane, uint32_t tacc,
                                              const TcRowInfo &ri, float *eb) {
    constexpr int NCH = NC / 32;
    const uint32_t tmem = tacc + ((uint32_t)(32 * quarter) << 16) + (uint32_t)c0;
    // vector stores need 16-byte (F32) / 8-byte (BF16) aligned row starts of C
    const int esz = e.c_dtype == SPREG_F32 ? 4 : 2;
    const bool vec_ok = (reinterpret_cast<uintptr_t>(e.C) % (4 * esz)) == 0 && (e.ldc % 4) == 0;
    int seg = 0;  // segment of the current column (coalesced products)
    if (e.nseg > 1 && ri.ok) {
        int lo2 = 0, hi2 = e.nseg - 1;
        while (lo2 < hi2) {
            const int mid = (lo2 + hi2 + 1) >> 1;
            if (e.seg_start[mid] <= n0 + c0) lo2 = mid;
            else hi2 = mid - 1;
        }
        seg = lo2;
    }
    uint32_t ra[32], rb[32];
    tc_ld32_issue(tmem, ra);
    tc_ld32_wait(ra);
#pragma unroll
    for (int ci = 0; ci < NCH; ++ci) {
        const int c = c0 + 32 * ci;
        if (ci + 1 < NCH) {
            if (ci & 1) tc_ld32_issue(tmem + (uint32_t)(32 * ci + 32), ra);
            else tc_ld32_issue(tmem + (uint32_t)(32 * ci + 32), rb);
        }
        if (ci & 1) tc_store_chunk<SPLIT>(e, n0, c, lane, rb, ri.rs, ri.ok, ri.orow, vec_ok, seg, eb);
        else tc_store_chunk<SPLIT>(e, n0, c, lane, ra, ri.rs, ri.ok, ri.orow, vec_ok, seg, eb);
        if (ci + 1 < NCH) {
            if (ci & 1) tc_ld32_wait(ra);
            else tc_ld32_wait(rb);
        }
    }
}

// Persistent.  CTA b takes output tiles b, b + gridDim.x, ...  Warp 0 (lane 0) loads the operand
// tiles of every K block of those tiles into the stage ring; warp 1 (lane 0) issues the MMAs of tile j
// into TMEM accumulator j % 2 (2 x BN columns) and commits "acc full"; warps 2..9 read an
// accumulator (warp w reads TMEM lane quarter w % 4, columns [BN / 2 * h, BN / 2 * (h + 1)) with
// h = (w - 2) / 4), store the tile and arrive on "acc empty", so the next tile's MMAs overlap this
// tile's stores.  Eight epilogue warps, two per SM sub-partition, hide the latency of the TMEM
// loads, shuffles and shared-memory transposes of the stores (four took longer per tile than the
// MMAs of a 512-deep tile).
//
// SPLIT: a stage holds [A hi | A lo | B hi | B lo]; per 16-deep K step the issuer runs
// hi.hi, hi.lo and lo.hi into the same accumulator (FP16 operands).
template <int BN, bool SPLIT>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_rows_kernel(const __grid_constant__ TcParams p, const int total_tiles) {
    constexpr int STAGES = tc_stages<BN, SPLIT>();
    constexpr int BK = tc_bk<SPLIT>();
    constexpr uint32_t TC_STAGE = tc_stage<BN, SPLIT>(), TC_TMEM_COLS = 2 * BN;
    constexpr uint32_t TILE_A = tc_tile_a<BN, SPLIT>();         // A hi -> A lo
    constexpr uint32_t A_BYTES = (SPLIT ? 2u : 1u) * TILE_A;     // B tiles start here
    constexpr uint32_t B_HALF = tc_tile_b<BN, SPLIT>();          // B hi -> B lo
    constexpr int TC_BN = BN;
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t sbase = (raw + 1023u) & ~1023u;  // the swizzle atoms need 1024-byte alignment
    const uint32_t bars = sbase + STAGES * TC_STAGE;
    const uint32_t full0 = bars, empty0 = bars + 8u * STAGES;
    const uint32_t accf0 = bars + 16u * STAGES, acce0 = accf0 + 16u;  // acc full / empty, 2 each
    const uint32_t tmem_slot = acce0 + 16u;
    float *const epi = reinterpret_cast<float *>(smem_raw + (bars + 256u - raw));  // epilogue staging buffers
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc_mbar_init(full0 + 8u * s, 1);
            tc_mbar_init(empty0 + 8u * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            tc_mbar_init(accf0 + 8u * a, 1);
            tc_mbar_init(acce0 + 8u * a, TC_EPI_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tmem_slot),
                     "r"(TC_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t tmem;
    asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(tmem_slot) : "memory");
    // output tile t of problem q
    auto tile_of = [&](const TcProblem &q, int t, int &m0, int &n0) {
        const int local = t - q.tile_begin;
        m0 = (local / q.tiles_n) * TC_BM;
        n0 = (local % q.tiles_n) * TC_BN;
    };

    if (warp == 0) {
        if (lane == 0) {
            // producer: operand tiles of every K block of every tile of this CTA
            int64_t g = 0;  // K blocks issued so far (stage g % STAGES)
            bool ok = true;
            int last_q = -1;
            for (int t = (int)blockIdx.x; t < total_tiles && ok; t += (int)gridDim.x) {
                const int qi = tc_problem_of(p, t);
                const TcProblem &q = p.prob[qi];
                if (qi != last_q) {
                    tc_map_acquire(q.a_map);
                    tc_map_acquire(q.b_map);
                    last_q = qi;
                }
                int m0, n0;
                tile_of(q, t, m0, n0);
                for (int kb = 0; kb < q.kblocks; ++kb, ++g) {
                    const int s = (int)(g % STAGES);
                    if (g >= STAGES && !tc_wait(empty0 + 8u * s, (uint32_t)(((g / STAGES) - 1) & 1), p.status, 21)) {
                        ok = false;
                        break;
                    }
                    const uint32_t st = sbase + (uint32_t)s * TC_STAGE;
                    tc_expect_tx(full0 + 8u * s, TC_STAGE);
                    const int kx = (q.kb0 + kb) * BK;  // K offset of this block
                    tc_tma_2d(st, q.a_map, kx, m0, full0 + 8u * s);
                    if constexpr (SPLIT) {
                        tc_tma_2d(st + TILE_A, q.a_map, kx, q.a_lo_row + m0, full0 + 8u * s);
                        // B halves, N-major: BN / 64 copies of 64 columns x 64 K rows each, 8 KB apart
#pragma unroll
                        for (int jb = 0; jb < TC_BN / 64; ++jb) {
                            tc_tma_2d(st + A_BYTES + 8192u * jb, q.b_map, n0 + 64 * jb, kx, full0 + 8u * s);
                            tc_tma_2d(st + A_BYTES + B_HALF + 8192u * jb, q.b_map, n0 + 64 * jb, q.b_lo_row + kx,
                                      full0 + 8u * s);
                        }
                    } else if (q.b_mn) {
                        // N-major B: BN / 64 copies of 64 columns x 64 K rows, 8 KB apart
#pragma unroll
                        for (int jb = 0; jb < TC_BN / 64; ++jb)
                            tc_tma_2d(st + A_BYTES + 8192u * jb, q.b_map, n0 + 64 * jb, kx, full0 + 8u * s);
                    } else {
                        tc_tma_2d(st + A_BYTES, q.b_map, kx, n0, full0 + 8u * s);
                    }
                }
            }
            // before the CTA can finish, every copy issued has landed
            const int64_t tail = g - STAGES > 0 ? g - STAGES : 0;
            for (int64_t k = tail; k < g; ++k)
                tc_wait(full0 + 8u * (uint32_t)(k % STAGES), (uint32_t)((k / STAGES) & 1), p.status, 22);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN, !SPLIT);
            int64_t g = 0;
            int j = 0;  // this CTA's tile count
            bool ok = true;
            for (int t = (int)blockIdx.x; t < total_tiles && ok; t += (int)gridDim.x, ++j) {
                const TcProblem &q = p.prob[tc_problem_of(p, t)];
                const int a = j & 1;
                if (j >= 2 && !tc_wait(acce0 + 8u * a, (uint32_t)(((j >> 1) - 1) & 1), p.status, 25)) break;
                tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(a * TC_BN);
                for (int kb = 0; kb < q.kblocks; ++kb, ++g) {
                    const int s = (int)(g % STAGES);
                    if (!tc_wait(full0 + 8u * s, (uint32_t)((g / STAGES) & 1), p.status, 23)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t st = sbase + (uint32_t)s * TC_STAGE;
                    if constexpr (SPLIT) {
                        // 128-byte swizzle; a 16-deep K step is 32 bytes into each A row and 16 rows of
                        // 128 bytes of B; N-major B (transpose-B bit of the instruction descriptor)
#pragma unroll
                        for (int k = 0; k < BK / 16; ++k) {
                            const uint64_t ah = tc_desc(st + 32u * k), bh = tc_desc_mn(st + A_BYTES + 2048u * k);
                            tc_mma(dacc, ah, bh, idesc | (1u << 16), (kb | k) != 0);
                            tc_mma(dacc, ah, tc_desc_mn(st + A_BYTES + B_HALF + 2048u * k), idesc | (1u << 16), 1);
                            tc_mma(dacc, tc_desc(st + TILE_A + 32u * k), bh, idesc | (1u << 16), 1);
                        }
                    } else if (q.b_mn) {
                        // N-major B (transpose-B bit of the instruction descriptor); a 16-deep K step is
                        // 16 rows of 128 bytes
#pragma unroll
                        for (int k = 0; k < BK / 16; ++k)
                            tc_mma(dacc, tc_desc(st + 32u * k), tc_desc_mn(st + A_BYTES + 2048u * k), idesc | (1u << 16),
                                   (kb | k) != 0);
                    } else {
#pragma unroll
                        for (int k = 0; k < BK / 16; ++k)
                            tc_mma(dacc, tc_desc(st + 32u * k), tc_desc(st + A_BYTES + 32u * k), idesc,
                                   (kb | k) != 0);
                    }
                    tc_commit(empty0 + 8u * s);  // the stage is free once these MMAs have read it
                }
                tc_commit(accf0 + 8u * a);  // accumulator a holds tile j once these MMAs complete
            }
        }
    } else {
        // epilogue warps 2..9
        const int quarter = warp & 3, half = (warp - 2) >> 2;
        int j = 0;
        bool ok = true;
        for (int t = (int)blockIdx.x; t < total_tiles; t += (int)gridDim.x, ++j) {
            const TcProblem &q = p.prob[tc_problem_of(p, t)];
            int m0, n0;
            tile_of(q, t, m0, n0);
            const TcRowInfo ri = tc_row_info<SPLIT>(q, m0, quarter, lane);  // before the accumulator is ready
            const int a = j & 1;
            ok = ok && __all_sync(0xffffffffu, tc_wait(accf0 + 8u * a, (uint32_t)((j >> 1) & 1), p.status, 24));
            tc_fence_after();
            if (!ok) break;
            const TcEpi e = tc_epi_of(q);
            tc_store_tile<BN / 2, SPLIT>(e, n0, half * (BN / 2), quarter, lane, tmem + (uint32_t)(a * TC_BN), ri,
                                         epi + (warp - 2) * (32 * 33));  // adds the lane quarter
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive_tc(acce0 + 8u * a);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
}

// FP32 -> (hi, lo) FP16 split with a power-of-two scale.  Exponent s with max * 2^s in [2^14, 2^15)
// (0 for a zero or non-finite max), clamped to [-126, 126] so that 2^s and 2^-s are normal floats.
__device__ __forceinline__ int split_exponent(float maxabs) {
    const uint32_t bits = __float_as_uint(maxabs);
    const int e = (int)((bits >> 23) & 0xFFu);
    if (maxabs == 0.0f || e == 0xFF) return 0;
    const int s = 14 - (e == 0 ? -126 : e - 127);  // max in [2^E, 2^(E+1)) for a normal max
    return s < -126 ? -126 : s > 126 ? 126 : s;
}
__device__ __forceinline__ float pow2f(int s) { return __uint_as_float((uint32_t)(s + 127) << 23); }
__device__ __forceinline__ void split_half(float x, __half &hi, __half &lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));  // x - hi is exact in FP32
}

// A rows of a split product: row i of a (FP32, lda) -> out row i (high halves) and out row rows + i
// (low halves), FP16, columns [k, ld_out) zero; inv_scale[i] = 2^-s of the row's scale.  One CTA per row.
__global__ void __launch_bounds__(256) split_rows_kernel(const float *__restrict__ a, int64_t lda, int64_t rows,
                                                          int64_t k, __half *__restrict__ out, int64_t ld_out,
                                                          float *__restrict__ inv_scale) {
    const int64_t i = blockIdx.x;
    const float *ar = a + i * lda;
    float m = 0.0f;
    for (int64_t c = threadIdx.x; c < k; c += 256) m = fmaxf(m, fabsf(ar[c]));
    __shared__ float red[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = red[0];
#pragma unroll
    for (int w = 1; w < 8; ++w) m = fmaxf(m, red[w]);
    const int s = split_exponent(m);
    const float sc = pow2f(s);
    if (threadIdx.x == 0) inv_scale[i] = pow2f(-s);
    __half *hi = out + i * ld_out, *lo = out + (rows + i) * ld_out;
    for (int64_t c = threadIdx.x; c < ld_out; c += 256) {
        __half h = __float2half_rn(0.0f), l = h;
        if (c < k) split_half(ar[c] * sc, h, l);
        hi[c] = h;
        lo[c] = l;
    }
}

// B of one split product (or one segment of coalesced products): FP32 k x n (row stride ldb) ->
// FP16 high halves at hi[r * ld + j] for r < k64 and low halves at hi[lo_off + r * ld + j], rows
// [k, k64) zero; inv_scale[j] = 2^-s of column j's scale.
struct SplitBItem {
    const float *b;
    int64_t ldb;
    __half *hi;
    int64_t ld, lo_off;
    float *inv_scale;
    int32_t k, n, k64, pad;
};

// One CTA of 16 warps per (64-column chunk, item): lane l of each warp takes columns 2l and 2l + 1 of
// the chunk, warp w the rows w, w + 16, ...  A column's maximum over k (shared-memory reduction over
// the warps), then the split.  RPT > 0 (k64 <= 16 RPT): each thread's RPT rows are loaded once, all
// in flight together, and stay in registers from the maximum to the split (one read of B); RPT = 0:
// two passes over B, eight rows' loads in flight per thread.
constexpr int SPLIT_WARPS = 16;
template <int RPT>
__global__ void __launch_bounds__(32 * SPLIT_WARPS) split_cols_kernel(const SplitBItem *__restrict__ items) {
    const SplitBItem it = items[blockIdx.y];
    const int j0 = blockIdx.x * 64;
    if (j0 >= it.n) return;  // uniform per block
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int j = j0 + 2 * lane;
    const bool c0 = j < it.n, c1 = j + 1 < it.n;
    const bool vec = ((reinterpret_cast<uintptr_t>(it.b) | (uintptr_t)(it.ldb * 4)) % 8) == 0;
    auto load2 = [&](int r, float &x0, float &x1) {
        x0 = x1 = 0.0f;
        if (r >= it.k) return;
        const float *row = it.b + (int64_t)r * it.ldb;
        if (vec && c1) {
            const float2 v = __ldg(reinterpret_cast<const float2 *>(row + j));
            x0 = v.x;
            x1 = v.y;
        } else {
            if (c0) x0 = __ldg(row + j);
            if (c1) x1 = __ldg(row + j + 1);
        }
    };
    constexpr int U = 8;                   // rows per unrolled iteration of a thread (RPT = 0)
    constexpr int STEP = U * SPLIT_WARPS;  // rows per unrolled iteration of the CTA
    float xs[RPT > 0 ? RPT : 1][2];
    float m0 = 0.0f, m1 = 0.0f;
    if constexpr (RPT > 0) {
#pragma unroll
        for (int u = 0; u < RPT; ++u) load2(w + u * SPLIT_WARPS, xs[u][0], xs[u][1]);
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
            m0 = fmaxf(m0, fabsf(xs[u][0]));
            m1 = fmaxf(m1, fabsf(xs[u][1]));
        }
    } else {
        for (int r = w; r < it.k; r += STEP) {
            float x[U][2];
#pragma unroll
            for (int u = 0; u < U; ++u) load2(r + u * SPLIT_WARPS, x[u][0], x[u][1]);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                m0 = fmaxf(m0, fabsf(x[u][0]));
                m1 = fmaxf(m1, fabsf(x[u][1]));
            }
        }
    }
    __shared__ float red[SPLIT_WARPS][64];
    red[w][2 * lane] = m0;
    red[w][2 * lane + 1] = m1;
    __syncthreads();
    m0 = red[0][2 * lane];
    m1 = red[0][2 * lane + 1];
#pragma unroll
    for (int v = 1; v < SPLIT_WARPS; ++v) {
        m0 = fmaxf(m0, red[v][2 * lane]);
        m1 = fmaxf(m1, red[v][2 * lane + 1]);
    }
    // (every warp reduces the same values; red is not written again)
    const int s0 = split_exponent(m0), s1 = split_exponent(m1);
    const float sc0 = pow2f(s0), sc1 = pow2f(s1);
    if (w == 0) {
        if (c0) it.inv_scale[j] = pow2f(-s0);
        if (c1) it.inv_scale[j + 1] = pow2f(-s1);
    }
    const bool vec_out = ((reinterpret_cast<uintptr_t>(it.hi + j0) | (uintptr_t)(it.ld * 2)) % 4) == 0;
    auto put = [&](int rr, float x0, float x1) {
        __half h0, l0, h1, l1;
        split_half(x0 * sc0, h0, l0);
        split_half(x1 * sc1, h1, l1);
        __half *hp = it.hi + (int64_t)rr * it.ld + j, *lp = hp + it.lo_off;
        if (vec_out && c1) {
            *reinterpret_cast<__half2 *>(hp) = __halves2half2(h0, h1);
            *reinterpret_cast<__half2 *>(lp) = __halves2half2(l0, l1);
        } else {
            if (c0) { hp[0] = h0; lp[0] = l0; }
            if (c1) { hp[1] = h1; lp[1] = l1; }
        }
    };
    if constexpr (RPT > 0) {
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
            const int rr = w + u * SPLIT_WARPS;
            if (rr < it.k64) put(rr, xs[u][0], xs[u][1]);
        }
    } else {
        for (int r = w; r < it.k64; r += STEP) {
            float x[U][2];
#pragma unroll
            for (int u = 0; u < U; ++u) load2(r + u * SPLIT_WARPS, x[u][0], x[u][1]);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int rr = r + u * SPLIT_WARPS;
                if (rr >= it.k64) break;
                put(rr, x[u][0], x[u][1]);
            }
        }
    }
}

// One B of a batched call: transposed into dst (n x K8, zero past k).
struct TransposeItem {
    const __nv_bfloat16 *b;
    __nv_bfloat16 *dst;
    int64_t ldb;
    int32_t k, n, K8, pad;
};

// All B of a batched call in one launch: Bt[j][k] = B[k][j] for k < K (zero up to K8), j < n, in
// 64 x 64 tiles through shared memory; blockIdx.z picks the item, x / y its tile.  Rows of B are
// read 16 bytes at a time when they are 16-byte aligned, rows of Bt are written 16 bytes at a time
// (K8 and the tile's K offset are multiples of 8).
__global__ void __launch_bounds__(256) transpose_items_kernel(const TransposeItem *__restrict__ items) {
    const TransposeItem it = items[blockIdx.z];
    const int k0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    if (k0 >= it.K8 || j0 >= it.n) return;  // uniform per block
    __shared__ uint16_t tile[64][66];        // [k][j]; a 33-word row stride spreads the column reads
    const uint16_t *B = reinterpret_cast<const uint16_t *>(it.b);
    const bool vec_in = ((reinterpret_cast<uintptr_t>(B) | (uintptr_t)(it.ldb * 2)) % 16) == 0;
    for (int c = threadIdx.x; c < 512; c += 256) {
        const int kr = c >> 3, jc = (c & 7) * 8;
        const int k = k0 + kr, j = j0 + jc;
        uint16_t v[8];
        if (k < it.k && vec_in && j + 8 <= it.n) {
            const uint4 w = *reinterpret_cast<const uint4 *>(B + (int64_t)k * it.ldb + j);
            const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                v[2 * e] = (uint16_t)(ws[e] & 0xFFFFu);
                v[2 * e + 1] = (uint16_t)(ws[e] >> 16);
            }
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = (k < it.k && j + e < it.n) ? B[(int64_t)k * it.ldb + j + e] : (uint16_t)0;
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) tile[kr][jc + e] = v[e];
    }
    __syncthreads();
    uint16_t *D = reinterpret_cast<uint16_t *>(it.dst);
    for (int c = threadIdx.x; c < 512; c += 256) {
        const int jr = c >> 3, kc = (c & 7) * 8;
        const int j = j0 + jr, k = k0 + kc;
        if (j >= it.n || k >= it.K8) continue;  // k + 8 <= K8: both are multiples of 8
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) w[e] = (uint32_t)tile[kc + 2 * e][jr] | ((uint32_t)tile[kc + 2 * e + 1][jr] << 16);
        *reinterpret_cast<uint4 *>(D + (int64_t)j * it.K8 + k) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tc_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *q = nullptr;
        cudaDriverEntryPointQueryResult r;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &q, 12000, cudaEnableDefault, &r) != cudaSuccess ||
            r != cudaDriverEntryPointSuccess)
            q = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(q);
    }();
    return fn;
}

// 16-bit matrix of `rows` x `cols` (row stride ld elements) as 64 x box_rows boxes (128-byte rows) with the
// 128-byte swizzle; FP16 (split products) or BF16.
int tc_map(CUtensorMap *map, const void *base, int64_t cols, int64_t rows, int64_t ld, int box_rows, bool f16) {
    auto enc = tc_encoder();
    SPREG_CHECK_ARG(enc, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    const cuuint32_t box[2] = {(cuuint32_t)(f16 ? TC_BK_SPLIT : TC_BK), (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                     const_cast<void *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SPREG_CHECK_ARG(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d) for a %lld x %lld 16-bit operand", (int)r,
                    (long long)rows, (long long)cols);
    return SPREG_OK;
}

// One product of either form, as the plan builder sees it.
struct TcItem {
    const void *a;         // BF16 rows (rows x lda), or the split pair (2 rows x lda, FP16)
    int64_t rows, k, lda;
    const int32_t *row_index;
    const float *row_scale;  // split: 2^-s per row
    const void *b;           // BF16 or (split) FP32, k x ldb
    int64_t ldb;
    void *c;
    int64_t ldc, n;
    int32_t c_dtype, load_c, epilogue, tile_n;
};

struct TcGroup {
    int32_t first;
    std::vector<int32_t> members;
    int64_t n = 0;
    int64_t buf_off = 0;     // Bt (transposed BF16) or the split B pair, in the scratch buffer
    int64_t scale_off = 0;   // split: column scales
    int64_t ldn = 0, k64 = 0;  // split: row stride of the B pair, K rounded up to 64
    int64_t seg_off = 0, seg_c_off = 0, seg_ldc_off = 0;  // segment tables (in the table)
    bool mn = false;         // B read as an N-major operand
};

struct TcLaunch {
    std::unique_ptr<TcParams> p;
    int bn = 128, tiles = 0;
};

// Everything one call (or one reusable plan) launches: the B preparation (transpose or split) and
// the tensor-core launches, with their device table.  Built in two phases: sizes, then -- once the
// scratch buffer exists -- pointers and tensor maps.
struct TcPlan {
    bool split = false;
    std::vector<TcItem> items;
    std::vector<TcGroup> groups;
    int64_t buf_bytes = 0, tab_base = 0, scratch_bytes = 0;
    std::vector<unsigned char> tab;
    int64_t prep_off = 0;                 // transpose / split items in the table
    int32_t nprep = 0;
    int64_t max_kt = 1, max_nt = 1;       // transpose grid
    int64_t max_ct = 1;                   // split grid: 64-column chunks
    int64_t max_k64 = 0;                  // split: the longest K (rounded up to 64) of the prepared B
    int64_t maps_off = 0;                 // 2 tensor maps per group
    std::vector<TcLaunch> launches;
    char *scratch = nullptr;
    int sms = 148;
};

int64_t tab_put(std::vector<unsigned char> &tab, const void *src, size_t len, size_t align = 8) {
    const size_t at = (tab.size() + align - 1) / align * align;
    tab.resize(at + (len + 7) / 8 * 8);
    if (src) memcpy(tab.data() + at, src, len);
    return (int64_t)at;
}

int tc_device_setup(int *sms_out) {
    static std::atomic<bool> configured[64];  // per device
    static std::atomic<int> sms_of[64];       // per device, 0 until queried
    int dev = 0;
    SPREG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !configured[dev].load()) {
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<128, false>()));
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<256, false>()));
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<128, true>()));
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<256, true>()));
        configured[dev].store(true);
    }
    if (dev >= 0 && dev < 64 && !sms_of[dev].load()) {
        int v = 0;
        SPREG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        sms_of[dev].store(v);
    }
    *sms_out = (dev >= 0 && dev < 64 && sms_of[dev].load() > 0) ? sms_of[dev].load() : 148;
    return SPREG_OK;
}

// Phase 1: checks, groups of coalesced products, scratch and table sizes.
int tc_plan_build(TcPlan &pl) {
    const bool split = pl.split;
    std::map<std::tuple<const void *, int64_t, int64_t, int64_t, const void *, int32_t, int32_t, int32_t>, size_t> key;
    for (int32_t i = 0; i < (int32_t)pl.items.size(); ++i) {
        const TcItem &it = pl.items[i];
        SPREG_CHECK_ARG(it.rows >= 0 && it.k >= 0 && it.n >= 0, "item %d: negative size", i);
        if (it.rows == 0 || it.n == 0) continue;
        SPREG_CHECK_ARG(it.a && it.row_index && it.c && it.b && (!split || it.row_scale), "item %d: null pointer", i);
        SPREG_CHECK_ARG(it.rows <= INT32_MAX / 2 && it.k <= INT32_MAX / 2 && it.n <= INT32_MAX, "item %d: size out of range",
                        i);
        SPREG_CHECK_ARG(it.c_dtype == SPREG_F32 || (!split && it.c_dtype == SPREG_BF16),
                        split ? "item %d: C must be F32" : "item %d: C must be F32 or BF16", i);
        SPREG_CHECK_ARG(it.epilogue == SPREG_EPILOGUE_NONE || it.epilogue == SPREG_EPILOGUE_RELU, "item %d: bad epilogue",
                        i);
        SPREG_CHECK_ARG(it.lda >= it.k && (it.lda * 2) % 16 == 0 && reinterpret_cast<uintptr_t>(it.a) % 16 == 0,
                        "A rows must be 16-byte aligned with a row stride of a multiple of 8 elements (item %d, lda "
                        "%lld)", i, (long long)it.lda);
        SPREG_CHECK_ARG(it.ldb >= it.n && it.ldc >= it.n, "item %d: ldb / ldc smaller than n", i);
        SPREG_CHECK_ARG(it.k > 0, "item %d: K must be positive", i);
        SPREG_CHECK_ARG(it.tile_n == 0 || it.tile_n == 128 || it.tile_n == 256, "item %d: tile_n must be 0, 128 or 256",
                        i);
        auto kk = std::make_tuple(it.a, it.rows, it.k, it.lda, (const void *)it.row_index, it.c_dtype,
                                  it.load_c ? 1 : 0, it.epilogue);
        auto f = key.find(kk);
        if (f == key.end()) {
            key.emplace(kk, pl.groups.size());
            TcGroup g;
            g.first = i;
            g.members.push_back(i);
            g.n = it.n;
            pl.groups.push_back(std::move(g));
        } else {
            TcGroup &g = pl.groups[f->second];
            g.members.push_back(i);
            g.n += it.n;
        }
    }
    // scratch: each group's Bt (n x K8) or split B pair (2 x K64 x ldn FP16) + column scales
    int64_t bytes = 0;
    for (TcGroup &g : pl.groups) {
        SPREG_CHECK_ARG(g.n <= INT32_MAX, "coalesced products wider than 2^31 columns");
        const TcItem &f = pl.items[g.first];
        if (split) {
            g.mn = true;
            g.k64 = (f.k + TC_BK - 1) / TC_BK * TC_BK;
            g.ldn = (g.n + 7) / 8 * 8;
            g.buf_off = bytes;
            bytes += (2 * g.k64 * g.ldn * 2 + 255) / 256 * 256;
            g.scale_off = bytes;
            bytes += (g.n * 4 + 255) / 256 * 256;
            continue;
        }
        g.mn = g.members.size() == 1 && reinterpret_cast<uintptr_t>(f.b) % 16 == 0 && (f.ldb * 2) % 16 == 0;
        if (g.mn) continue;
        const int64_t K8 = (f.k + 7) / 8 * 8;
        g.buf_off = bytes;
        bytes += (g.n * K8 * 2 + 255) / 256 * 256;
    }
    pl.buf_bytes = bytes;
    // table: tensor maps, segment tables, preparation items (pointers filled in phase 2)
    pl.tab.clear();
    pl.maps_off = tab_put(pl.tab, nullptr, 2 * sizeof(CUtensorMap) * pl.groups.size(), 128);
    for (TcGroup &g : pl.groups) {
        if (g.members.size() < 2) continue;
        std::vector<int32_t> starts;
        int32_t o = 0;
        for (int32_t m : g.members) {
            starts.push_back(o);
            o += (int32_t)pl.items[m].n;
        }
        starts.push_back(o);
        g.seg_off = tab_put(pl.tab, starts.data(), starts.size() * 4);
        g.seg_c_off = tab_put(pl.tab, nullptr, g.members.size() * 8);
        g.seg_ldc_off = tab_put(pl.tab, nullptr, g.members.size() * 8);
    }
    pl.nprep = 0;
    for (const TcGroup &g : pl.groups) {
        if (g.mn && !split) continue;
        for (int32_t m : g.members) {
            ++pl.nprep;
            const TcItem &it = pl.items[m];
            if (split) {
                pl.max_ct = std::max<int64_t>(pl.max_ct, (it.n + 63) / 64);
                pl.max_k64 = std::max<int64_t>(pl.max_k64, g.k64);
            } else {
                pl.max_kt = std::max<int64_t>(pl.max_kt, ((it.k + 7) / 8 * 8 + 63) / 64);
                pl.max_nt = std::max<int64_t>(pl.max_nt, (it.n + 63) / 64);
            }
        }
    }
    SPREG_CHECK_ARG(pl.nprep <= 65535 && pl.max_nt <= 65535 && pl.max_ct <= INT32_MAX, "too many products in one call");
    pl.prep_off = tab_put(pl.tab, nullptr, (size_t)pl.nprep * (split ? sizeof(SplitBItem) : sizeof(TransposeItem)));
    pl.tab_base = (pl.buf_bytes + 255) / 256 * 256;
    pl.scratch_bytes = pl.tab_base + (int64_t)pl.tab.size() + 16;
    return SPREG_OK;
}

// Phase 2 (scratch allocated): preparation items, segment tables, tensor maps, launch parameters.
int tc_plan_fill(TcPlan &pl, int *status) {
    const bool split = pl.split;
    char *const scratch = pl.scratch;
    char *const tabd = scratch + pl.tab_base;
    int st = SPREG_OK;
    // preparation items and segment tables
    {
        int32_t t = 0;
        for (TcGroup &g : pl.groups) {
            if (g.members.size() > 1) {
                std::vector<uint64_t> cs;
                std::vector<int64_t> lds;
                for (int32_t m : g.members) {
                    cs.push_back(reinterpret_cast<uint64_t>(pl.items[m].c));
                    lds.push_back(pl.items[m].ldc);
                }
                memcpy(pl.tab.data() + g.seg_c_off, cs.data(), cs.size() * 8);
                memcpy(pl.tab.data() + g.seg_ldc_off, lds.data(), lds.size() * 8);
            }
            if (g.mn && !split) continue;
            int64_t o = 0;  // column offset of the member in its group
            for (int32_t m : g.members) {
                const TcItem &it = pl.items[m];
                if (split) {
                    SplitBItem si;
                    si.b = static_cast<const float *>(it.b);
                    si.ldb = it.ldb;
                    si.hi = reinterpret_cast<__half *>(scratch + g.buf_off) + o;
                    si.ld = g.ldn;
                    si.lo_off = g.k64 * g.ldn;
                    si.inv_scale = reinterpret_cast<float *>(scratch + g.scale_off) + o;
                    si.k = (int32_t)it.k;
                    si.n = (int32_t)it.n;
                    si.k64 = (int32_t)g.k64;
                    si.pad = 0;
                    memcpy(pl.tab.data() + pl.prep_off + sizeof(SplitBItem) * t, &si, sizeof si);
                } else {
                    const int64_t K8 = (pl.items[g.first].k + 7) / 8 * 8;
                    TransposeItem ti;
                    ti.b = static_cast<const __nv_bfloat16 *>(it.b);
                    ti.dst = reinterpret_cast<__nv_bfloat16 *>(scratch + g.buf_off) + o * K8;
                    ti.ldb = it.ldb;
                    ti.k = (int32_t)it.k;
                    ti.n = (int32_t)it.n;
                    ti.K8 = (int32_t)K8;
                    ti.pad = 0;
                    memcpy(pl.tab.data() + pl.prep_off + sizeof(TransposeItem) * t, &ti, sizeof ti);
                }
                ++t;
                o += it.n;
            }
        }
    }
    // tensor maps (device table) and launches of up to TC_MAX_PROBLEMS problems
    CUtensorMap *maps_h = reinterpret_cast<CUtensorMap *>(pl.tab.data() + pl.maps_off);
    const CUtensorMap *maps_d = reinterpret_cast<const CUtensorMap *>(tabd + pl.maps_off);
    pl.launches.clear();
    // (group, pass) problems: a split product of K > TC_SPLIT_CHUNK runs as passes over K chunks, pass
    // p in the launches after those of pass p - 1 (each pass adds into C); every other product is one
    // pass.  The maps of a group serve all its passes.
    std::vector<std::pair<int, int>> specs;
    int passes = 1;
    for (const TcGroup &g : pl.groups)
        passes = std::max<int>(passes, split ? (int)((pl.items[g.first].k + TC_SPLIT_CHUNK - 1) / TC_SPLIT_CHUNK) : 1);
    std::vector<size_t> pass_begin;
    for (int ps = 0; ps < passes; ++ps) {
        pass_begin.push_back(specs.size());
        for (size_t gi = 0; gi < pl.groups.size(); ++gi) {
            const int64_t k = pl.items[pl.groups[gi].first].k;
            if ((int64_t)ps * (split ? TC_SPLIT_CHUNK : k) < k) specs.emplace_back((int)gi, ps);
        }
    }
    pass_begin.push_back(specs.size());
    std::vector<std::pair<size_t, size_t>> chunks;  // [first, first + cnt) of specs, within one pass
    for (int ps = 0; ps < passes; ++ps)
        for (size_t f = pass_begin[ps]; f < pass_begin[ps + 1]; f += TC_MAX_PROBLEMS)
            chunks.emplace_back(f, std::min<size_t>(TC_MAX_PROBLEMS, pass_begin[ps + 1] - f));
    for (const auto &ch : chunks) {
        const size_t first = ch.first, cnt = ch.second;
        TcLaunch L;
        L.p.reset(new TcParams);
        TcParams &p = *L.p;
        memset(&p, 0, sizeof p);
        p.status = status;
        p.nprob = (int32_t)cnt;
        // Output tile width: as an item asks, else 128 when a problem is 128 columns or narrower, else
        // 256 -- unless the launch has at most two waves of 256-wide tiles and 128-wide ones take
        // fewer waves, a 128-wide tile counted as 0.6 of a 256-wide one (at K = 512 the same split
        // products ran 110.5 us in 128-wide tiles against 106.3 us in half as many 256-wide ones; at
        // long K the narrow tiles cost relatively more: a 4096^3 BF16 product ran 149 us in 1024
        // 128-wide tiles against 98 us in 512 256-wide ones).  A single wide product then takes
        // 128-wide tiles when its 256-wide tiles leave most of a last wave idle.
        int64_t min_n = INT64_MAX, tiles128 = 0, tiles256 = 0;
        int hint = 0;
        for (size_t j = 0; j < cnt; ++j) {
            const TcGroup &g = pl.groups[specs[first + j].first];
            const int64_t mt = (pl.items[g.first].rows + TC_BM - 1) / TC_BM;
            min_n = std::min<int64_t>(min_n, g.n);
            tiles128 += mt * ((g.n + 127) / 128);
            tiles256 += mt * ((g.n + 255) / 256);
            for (int32_t m : g.members)
                if (!hint && (pl.items[m].tile_n == 128 || pl.items[m].tile_n == 256)) hint = pl.items[m].tile_n;
        }
        const int64_t sms = pl.sms > 0 ? pl.sms : 148;
        const bool narrow = tiles256 <= 2 * sms &&
                            0.6 * (double)((tiles128 + sms - 1) / sms) < (double)((tiles256 + sms - 1) / sms);
        const int bn = hint ? hint : (min_n <= 128 || narrow ? 128 : 256);
        int64_t tiles = 0;
        for (size_t j = 0; j < cnt; ++j) {
            const size_t gi = (size_t)specs[first + j].first;
            const int ps = specs[first + j].second;
            const TcGroup &g = pl.groups[gi];
            const TcItem &it = pl.items[g.first];
            TcProblem &q = p.prob[j];
            q.a_map = maps_d + 2 * gi;
            q.b_map = maps_d + 2 * gi + 1;
            q.row_index = it.row_index;
            q.C = it.c;
            q.ldc = it.ldc;
            q.R = (int32_t)it.rows;
            q.n = (int32_t)g.n;
            const int64_t k0 = split ? (int64_t)ps * TC_SPLIT_CHUNK : 0;
            const int64_t kc = split ? std::min<int64_t>(TC_SPLIT_CHUNK, it.k - k0) : it.k;
            const bool last = k0 + kc >= it.k;
            const int64_t bk = split ? TC_BK_SPLIT : TC_BK;  // the kernel's K block
            q.kb0 = (int32_t)(k0 / bk);
            q.kblocks = (int32_t)((kc + bk - 1) / bk);
            q.c_dtype = it.c_dtype;
            q.load_c = (it.load_c || ps > 0) ? 1 : 0;
            q.epilogue = last ? it.epilogue : SPREG_EPILOGUE_NONE;
            q.nseg = (int32_t)g.members.size();
            if (q.nseg > 1) {
                q.seg_start = reinterpret_cast<const int32_t *>(tabd + g.seg_off);
                q.seg_c = reinterpret_cast<void *const *>(tabd + g.seg_c_off);
                q.seg_ldc = reinterpret_cast<const int64_t *>(tabd + g.seg_ldc_off);
            }
            q.tiles_n = (int32_t)((g.n + bn - 1) / bn);
            q.tile_begin = (int32_t)tiles;
            tiles += (it.rows + TC_BM - 1) / TC_BM * q.tiles_n;
            q.b_mn = g.mn ? 1 : 0;
            if (ps > 0) {  // later pass of a split product: the maps exist
                q.a_lo_row = (int32_t)it.rows;
                q.b_lo_row = (int32_t)g.k64;
                q.row_scale = it.row_scale;
                q.col_scale = reinterpret_cast<const float *>(scratch + g.scale_off);
            } else if (split) {
                q.a_lo_row = (int32_t)it.rows;
                q.b_lo_row = (int32_t)g.k64;
                q.row_scale = it.row_scale;
                q.col_scale = reinterpret_cast<const float *>(scratch + g.scale_off);
                if ((st = tc_map(&maps_h[2 * gi], it.a, it.k, 2 * it.rows, it.lda, TC_BM, true)) ||
                    (st = tc_map(&maps_h[2 * gi + 1], scratch + g.buf_off, g.n, 2 * g.k64, g.ldn, TC_BK_SPLIT, true)))
                    return st;
            } else {
                const int64_t K8 = (it.k + 7) / 8 * 8;
                if ((st = tc_map(&maps_h[2 * gi], it.a, it.k, it.rows, it.lda, TC_BM, false)) ||
                    (st = g.mn ? tc_map(&maps_h[2 * gi + 1], it.b, g.n, it.k, it.ldb, 64, false)
                               : tc_map(&maps_h[2 * gi + 1], scratch + g.buf_off, it.k, g.n, K8, bn, false)))
                    return st;
            }
        }
        SPREG_CHECK_ARG(tiles <= INT32_MAX, "too many output tiles in one launch");
        L.bn = bn;
        L.tiles = (int)tiles;
        pl.launches.push_back(std::move(L));
    }
    return SPREG_OK;
}

// Device table upload (stream-ordered copy of the host image).
int tc_plan_upload(const TcPlan &pl, cudaStream_t stream) {
    cudaError_t e = cudaMemcpyAsync(pl.scratch + pl.tab_base, pl.tab.data(), pl.tab.size(), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "tensor-core set-up: %s", cudaGetErrorString(e));
    return SPREG_OK;
}

template <int BN, bool SPLIT>
cudaError_t tc_launch(const TcParams &p, int tiles, int sms, cudaStream_t stream) {
    tc_rows_kernel<BN, SPLIT><<<(unsigned)std::min(tiles, sms), TC_THREADS, tc_smem<BN, SPLIT>(), stream>>>(p, tiles);
    return cudaGetLastError();
}

// The B preparation, then every tensor-core launch.
int tc_plan_launch(const TcPlan &pl, cudaStream_t stream) {
    cudaError_t e = cudaSuccess;
    const char *tabd = pl.scratch + pl.tab_base;
    if (pl.nprep > 0) {
        if (pl.split)
        {
            // rows of a column block held in registers when K is short (one read of B)
            const dim3 grid((unsigned)pl.max_ct, (unsigned)pl.nprep);
            const SplitBItem *items = reinterpret_cast<const SplitBItem *>(tabd + pl.prep_off);
            if (pl.max_k64 <= 16 * SPLIT_WARPS) split_cols_kernel<16><<<grid, 32 * SPLIT_WARPS, 0, stream>>>(items);
            else if (pl.max_k64 <= 32 * SPLIT_WARPS) split_cols_kernel<32><<<grid, 32 * SPLIT_WARPS, 0, stream>>>(items);
            else split_cols_kernel<0><<<grid, 32 * SPLIT_WARPS, 0, stream>>>(items);
        }
        else
            transpose_items_kernel<<<dim3((unsigned)pl.max_kt, (unsigned)pl.max_nt, (unsigned)pl.nprep), 256, 0,
                                     stream>>>(reinterpret_cast<const TransposeItem *>(tabd + pl.prep_off));
        e = cudaGetLastError();
    }
    for (size_t i = 0; i < pl.launches.size() && e == cudaSuccess; ++i) {
        const TcLaunch &L = pl.launches[i];
        if (L.tiles == 0) continue;
        if (pl.split)
            e = L.bn == 256 ? tc_launch<256, true>(*L.p, L.tiles, pl.sms, stream)
                            : tc_launch<128, true>(*L.p, L.tiles, pl.sms, stream);
        else
            e = L.bn == 256 ? tc_launch<256, false>(*L.p, L.tiles, pl.sms, stream)
                            : tc_launch<128, false>(*L.p, L.tiles, pl.sms, stream);
    }
    if (e != cudaSuccess) SPREG_FAIL(SPREG_ERR_CUDA, "tensor-core launch: %s", cudaGetErrorString(e));
    return SPREG_OK;
}

// One call: plan, stream-ordered scratch, upload, launch, stream-ordered free.
int tc_run_once(TcPlan &pl, cudaStream_t stream) {
    int st = tc_plan_build(pl);
    if (st) return st;
    if (pl.groups.empty()) return SPREG_OK;
    int *status = device_status_word(&st);
    if (st) return st;
    if ((st = tc_device_setup(&pl.sms))) return st;
    SPREG_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&pl.scratch), (size_t)pl.scratch_bytes, stream));
    if (!(st = tc_plan_fill(pl, status)) && !(st = tc_plan_upload(pl, stream))) st = tc_plan_launch(pl, stream);
    cudaFreeAsync(pl.scratch, stream);
    pl.scratch = nullptr;
    return st;
}

TcItem from_bf16(const spreg_dense_rows_item &it) {
    TcItem t;
    t.a = it.a_rows;
    t.rows = it.rows;
    t.k = it.k;
    t.lda = it.lda;
    t.row_index = it.row_index;
    t.row_scale = nullptr;
    t.b = it.b;
    t.ldb = it.ldb;
    t.c = it.c;
    t.ldc = it.ldc;
    t.n = it.n;
    t.c_dtype = it.c_dtype;
    t.load_c = it.load_c;
    t.epilogue = it.epilogue;
    t.tile_n = it.tile_n;
    return t;
}

TcItem from_f32(const spreg_dense_rows_f32_item &it) {
    TcItem t;
    t.a = it.a_split;
    t.rows = it.rows;
    t.k = it.k;
    t.lda = it.ld_split;
    t.row_index = it.row_index;
    t.row_scale = it.row_scale;
    t.b = it.b;
    t.ldb = it.ldb;
    t.c = it.c;
    t.ldc = it.ldc;
    t.n = it.n;
    t.c_dtype = SPREG_F32;
    t.load_c = it.load_c;
    t.epilogue = it.epilogue;
    t.tile_n = it.tile_n;
    return t;
}

}  // namespace

int dense_rows_batched_impl(const spreg_dense_rows_item *items, int32_t count, cudaStream_t stream) {
    SPREG_CHECK_ARG(count >= 0 && (count == 0 || items), "bad item list");
    TcPlan pl;
    pl.split = false;
    for (int32_t i = 0; i < count; ++i) pl.items.push_back(from_bf16(items[i]));
    return tc_run_once(pl, stream);
}

int dense_rows_bf16_impl(const void *a_rows, int64_t R, int64_t K, int64_t lda, const int32_t *row_index,
                         const void *b, int64_t ldb, void *c, int64_t ldc, int64_t n, int32_t c_dtype, int32_t load_c,
                         int32_t epilogue, cudaStream_t stream) {
    const spreg_dense_rows_item it = {a_rows, R, K, lda, row_index, b, ldb, c, ldc, n, c_dtype, load_c, epilogue, 0};
    return dense_rows_batched_impl(&it, 1, stream);
}

int dense_rows_f32_batched_impl(const spreg_dense_rows_f32_item *items, int32_t count, cudaStream_t stream) {
    SPREG_CHECK_ARG(count >= 0 && (count == 0 || items), "bad item list");
    TcPlan pl;
    pl.split = true;
    for (int32_t i = 0; i < count; ++i) pl.items.push_back(from_f32(items[i]));
    return tc_run_once(pl, stream);
}

int split_rows_f32_impl(const float *a_rows, int64_t rows, int64_t k, int64_t lda, void *a_split, int64_t ld_split,
                        float *row_scale, cudaStream_t stream) {
    SPREG_CHECK_ARG(rows >= 0 && k >= 0, "negative size");
    if (rows == 0) return SPREG_OK;
    SPREG_CHECK_ARG(a_rows && a_split && row_scale, "null pointer");
    SPREG_CHECK_ARG(lda >= k && ld_split >= k && ld_split % 8 == 0 && reinterpret_cast<uintptr_t>(a_split) % 16 == 0,
                    "the split pair needs a 16-byte aligned base and a row stride of a multiple of 8 elements >= k "
                    "(ld_split %lld, k %lld)", (long long)ld_split, (long long)k);
    SPREG_CHECK_ARG(rows <= INT32_MAX / 2, "too many rows");
    split_rows_kernel<<<(unsigned)rows, 256, 0, stream>>>(a_rows, lda, rows, k, static_cast<__half *>(a_split),
                                                         ld_split, row_scale);
    SPREG_CUDA(cudaGetLastError());
    return SPREG_OK;
}

// Reusable plan of FP32-accurate products: everything but the launches is done once (scratch, tensor
// maps, device table), so a run is two kernel launches with no host-side preparation.
struct TcPlanHandle {
    TcPlan pl;
    int device = -1;
};

namespace {

int tc_plan_create(TcPlanHandle *h, void **out, cudaStream_t stream) {
    TcPlan &pl = h->pl;
    int st = tc_plan_build(pl);
    int *status = nullptr;
    if (!st && !pl.groups.empty()) status = device_status_word(&st);
    if (!st) st = tc_device_setup(&pl.sms);
    if (!st) {
        cudaError_t e = cudaGetDevice(&h->device);
        if (e == cudaSuccess && !pl.groups.empty()) e = cudaMalloc(reinterpret_cast<void **>(&pl.scratch), (size_t)pl.scratch_bytes);
        if (e != cudaSuccess) {
            set_error(std::string("tensor-core plan: ") + cudaGetErrorString(e));
            st = e == cudaErrorMemoryAllocation ? SPREG_ERR_NOMEM : SPREG_ERR_CUDA;
        }
    }
    if (!st && !pl.groups.empty()) st = tc_plan_fill(pl, status);
    if (!st && !pl.groups.empty()) st = tc_plan_upload(pl, stream);
    if (!st && !pl.groups.empty()) {
        cudaError_t e = cudaStreamSynchronize(stream);  // the host image may change with the next build
        if (e != cudaSuccess) {
            set_error(std::string("tensor-core plan: ") + cudaGetErrorString(e));
            st = SPREG_ERR_CUDA;
        }
    }
    if (st) {
        if (pl.scratch) cudaFree(pl.scratch);
        delete h;
        return st;
    }
    *out = h;
    return SPREG_OK;
}

}  // namespace

int tc_plan_create_f32_impl(const spreg_dense_rows_f32_item *items, int32_t count, void **out, cudaStream_t stream) {
    SPREG_CHECK_ARG(out && count >= 0 && (count == 0 || items), "bad arguments");
    *out = nullptr;
    auto *h = new TcPlanHandle;
    h->pl.split = true;
    for (int32_t i = 0; i < count; ++i) h->pl.items.push_back(from_f32(items[i]));
    return tc_plan_create(h, out, stream);
}

int tc_plan_create_bf16_impl(const spreg_dense_rows_item *items, int32_t count, void **out, cudaStream_t stream) {
    SPREG_CHECK_ARG(out && count >= 0 && (count == 0 || items), "bad arguments");
    *out = nullptr;
    auto *h = new TcPlanHandle;
    h->pl.split = false;
    for (int32_t i = 0; i < count; ++i) h->pl.items.push_back(from_bf16(items[i]));
    return tc_plan_create(h, out, stream);
}

int tc_plan_run_impl(const void *plan, cudaStream_t stream) {
    SPREG_CHECK_ARG(plan, "null plan");
    const TcPlanHandle *h = static_cast<const TcPlanHandle *>(plan);
    if (h->pl.groups.empty()) return SPREG_OK;
    int dev = -1;
    SPREG_CUDA(cudaGetDevice(&dev));
    SPREG_CHECK_ARG(dev == h->device, "the plan was made on device %d, the current device is %d", h->device, dev);
    return tc_plan_launch(h->pl, stream);
}

void tc_plan_destroy_impl(void *plan) {
    if (!plan) return;
    auto *h = static_cast<TcPlanHandle *>(plan);
    if (h->pl.scratch) cudaFree(h->pl.scratch);
    delete h;
}

}  // namespace spreg
