// dense_tc.cu -- dense row panels on the 5th-generation tensor cores (tcgen05 MMA, tensor memory,
// TMA).
//
// C[row_index[i], 0:n] (+)= A_rows[i, 0:K] . B[0:K, 0:n] for the rows of a pruned matrix whose panels
// are dense enough that a BF16 tensor-core product beats the register-tiled executors.  BF16 operands,
// FP32 accumulation in tensor memory (TMEM), FP32 or BF16 output with load_c and the ReLU epilogue.
//
// One launch runs up to 80 such products ("problems", a tensor map pair each in the kernel
// parameters).  Its output tiles (128 rows x BN columns; BN 256 when every product of the launch has
// more than 128 columns, else 128) are shared out over persistent CTAs of 6 warps, at most one per
// SM, each finding a tile's problem by a binary search over the problems' first tiles:
//   * warp 0 (one lane) loads 64-deep K blocks of A_rows (128 x 64, K-major) and of B into a ring of
//     4 stages with 2-D tensor copies (TMA, 128-byte swizzle; "full" mbarriers with expected bytes).
//     A single product's B is read in place as an N-major operand (BN / 64 copies of 64 columns x
//     64 K rows); products coalesced over several B are first transposed into one K-major buffer;
//   * warp 1 (one lane) issues four tcgen05.mma.kind::f16 (M 128, N BN, K 16) per K block into one
//     of two TMEM accumulators, tcgen05.commit releasing the stage ("empty") and, per tile, the
//     accumulator ("acc full");
//   * warps 2-5 each read one 32-lane quarter of the accumulator with tcgen05.ld (the tile's rows),
//     apply load_c / ReLU, store through the row index (and the segment table of coalesced products)
//     and release the accumulator ("acc empty"), so the next tile's MMAs overlap these stores.
// Launches with at least a full wave of work run as clusters of 2 CTAs (spreg_tc_set_cluster): a pair
// computes two row blocks of one column block and each CTA loads its A tile and half of the B tile,
// multicast into both CTAs, so a B tile leaves L2 once per pair (tc_rows_kernel<BN, 2>).
// Rows past R and columns past n are zero-filled by the tensor copies and never stored; K past the
// end of A_rows / Bt reads as zero.  Every wait is bounded: a wait that gives up records a code in
// the device status word; TMEM is released on every path.
#include "spreg_common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

namespace spreg {

int *device_status_word(int *st);  // exec.cu

namespace {

constexpr int TC_BM = 128, TC_BK = 64, TC_STAGES = 4;
constexpr uint32_t TC_TILE_A = TC_BM * TC_BK * 2;  // 16 KB
// Output tile width BN (128 or 256): the MMA's N, the TMEM accumulator's columns, B tile rows.
template <int BN> constexpr uint32_t tc_tile_b() { return (uint32_t)BN * TC_BK * 2; }
template <int BN> constexpr uint32_t tc_stage() { return TC_TILE_A + tc_tile_b<BN>(); }
template <int BN> constexpr size_t tc_smem() {
    return 1024 /* alignment slack */ + TC_STAGES * tc_stage<BN>() + 256 /* barriers, TMEM slot */;
}

constexpr int TC_MAX_PROBLEMS = 80;  // problems per launch (two tensor maps each; parameters <= 32 KB)

struct TcProblem {
    CUtensorMap a_map;           // A_rows: columns [0, K) x rows [0, R), box 64 x 128, 128-byte swizzle
    CUtensorMap b_map;           // Bt: columns [0, K) x rows [0, n), box 64 x BN, 128-byte swizzle; or
                                 // (b_mn) B itself: columns [0, n) x rows [0, K), box 64 x 64
    const int32_t *row_index;    // output row of each A row
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
    int32_t b_mn;                // B read in place (N-major operand), no transpose
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
__device__ __forceinline__ void tc_tma_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

// The same copy delivered to every CTA of `mask` in the cluster: the data lands at offset dst of each
// CTA's shared memory and each CTA's barrier at offset bar receives the completed bytes.
__device__ __forceinline__ void tc_tma_2d_mc(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar,
                                             uint16_t mask) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster "
                 "[%0], [%1, {%2, %3}], [%4], %5;"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar), "h"(mask) : "memory");
}
__device__ __forceinline__ uint32_t tc_cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t tc_cluster_id() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t tc_cluster_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
// All threads of all CTAs of the cluster (every thread reaches it once, right after the set-up).
__device__ __forceinline__ void tc_cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Arrive on the barrier at offset bar of CTA `cta` of the cluster.
__device__ __forceinline__ void tc_remote_arrive(uint32_t bar, uint32_t cta) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(bar), "r"(cta));
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(r) : "memory");
}
__device__ __forceinline__ bool tc_wait_cluster(uint32_t bar, uint32_t phase, int *status, int code) {
    for (uint32_t it = 0; it < (1u << 22); ++it) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
        if (ok) return true;
    }
    if (status) atomicCAS(status, 0, code);
    return false;
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

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// The same arrival on the barrier at offset bar of every CTA of `mask` in the cluster.
__device__ __forceinline__ void tc_commit_mc(uint32_t bar, uint16_t mask) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(bar), "h"(mask) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
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

// Epilogue of one output tile by one warp: TMEM lanes 32 * quarter .. + 31 (tile rows) of the
// accumulator at TMEM address tacc (lane 0, its first column); load_c / ReLU; store through the
// row index (and segments).
template <int BN>
__device__ __forceinline__ void tc_store_tile(const TcProblem &q, int m0, int n0, int quarter, int lane, uint32_t tacc,
                                              bool ok) {
    constexpr int TC_BN = BN;
    const int r = m0 + 32 * quarter + lane;
    const bool row_ok = ok && r < q.R;
    const int64_t orow = row_ok ? q.row_index[r] : 0;
    const uint32_t tmem = tacc;
    const int warp = quarter;
    // vector stores need 16-byte (F32) / 8-byte (BF16) aligned row starts of C
    const int esz = q.c_dtype == SPREG_F32 ? 4 : 2;
    const bool vec_ok = (reinterpret_cast<uintptr_t>(q.C) % (4 * esz)) == 0 && (q.ldc % 4) == 0;
    if (ok) {
        int seg = 0;  // segment of the current column (coalesced products)
        if (q.nseg > 1 && row_ok) {
            int lo2 = 0, hi2 = q.nseg - 1;
            while (lo2 < hi2) {
                const int mid = (lo2 + hi2 + 1) >> 1;
                if (q.seg_start[mid] <= n0) lo2 = mid;
                else hi2 = mid - 1;
            }
            seg = lo2;
        }
        for (int c = 0; c < TC_BN; c += 16) {
            float v[16];
            tc_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);  // every lane takes part
            if (!row_ok) continue;
            if (q.nseg <= 1 && vec_ok && n0 + c + 16 <= q.n) {
                // whole 16-column chunk of one output: 16-byte (F32) / 8-byte (BF16) stores
                if (q.c_dtype == SPREG_F32) {
                    float4 *cp = reinterpret_cast<float4 *>(reinterpret_cast<float *>(q.C) + orow * q.ldc + n0 + c);
#pragma unroll
                    for (int j4 = 0; j4 < 4; ++j4) {
                        float4 o = make_float4(v[4 * j4], v[4 * j4 + 1], v[4 * j4 + 2], v[4 * j4 + 3]);
                        if (q.load_c) {
                            const float4 ci = cp[j4];
                            o.x += ci.x; o.y += ci.y; o.z += ci.z; o.w += ci.w;
                        }
                        if (q.epilogue == SPREG_EPILOGUE_RELU) {
                            o.x = fmaxf(o.x, 0.0f); o.y = fmaxf(o.y, 0.0f); o.z = fmaxf(o.z, 0.0f); o.w = fmaxf(o.w, 0.0f);
                        }
                        cp[j4] = o;
                    }
                } else {
                    uint2 *cp = reinterpret_cast<uint2 *>(reinterpret_cast<__nv_bfloat16 *>(q.C) + orow * q.ldc + n0 + c);
#pragma unroll
                    for (int j4 = 0; j4 < 4; ++j4) {
                        float o[4] = {v[4 * j4], v[4 * j4 + 1], v[4 * j4 + 2], v[4 * j4 + 3]};
                        if (q.load_c) {
                            const uint2 ci = cp[j4];
                            const __nv_bfloat162 c01 = *reinterpret_cast<const __nv_bfloat162 *>(&ci.x);
                            const __nv_bfloat162 c23 = *reinterpret_cast<const __nv_bfloat162 *>(&ci.y);
                            o[0] += __low2float(c01); o[1] += __high2float(c01);
                            o[2] += __low2float(c23); o[3] += __high2float(c23);
                        }
                        if (q.epilogue == SPREG_EPILOGUE_RELU)
                            for (int t = 0; t < 4; ++t) o[t] = fmaxf(o[t], 0.0f);
                        __nv_bfloat162 w01 = __floats2bfloat162_rn(o[0], o[1]), w23 = __floats2bfloat162_rn(o[2], o[3]);
                        uint2 w;
                        w.x = *reinterpret_cast<uint32_t *>(&w01);
                        w.y = *reinterpret_cast<uint32_t *>(&w23);
                        cp[j4] = w;
                    }
                }
                continue;
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = n0 + c + j;
                if (col >= q.n) break;
                void *cbase = q.C;
                int64_t ldc = q.ldc;
                int lcol = col;
                if (q.nseg > 1) {
                    while (col >= q.seg_start[seg + 1]) ++seg;
                    cbase = q.seg_c[seg];
                    ldc = q.seg_ldc[seg];
                    lcol = col - q.seg_start[seg];
                }
                float o = v[j];
                if (q.c_dtype == SPREG_F32) {
                    float *cp = reinterpret_cast<float *>(cbase) + orow * ldc + lcol;
                    if (q.load_c) o += *cp;
                    if (q.epilogue == SPREG_EPILOGUE_RELU) o = fmaxf(o, 0.0f);
                    *cp = o;
                } else {
                    __nv_bfloat16 *cp = reinterpret_cast<__nv_bfloat16 *>(cbase) + orow * ldc + lcol;
                    if (q.load_c) o += __bfloat162float(*cp);
                    if (q.epilogue == SPREG_EPILOGUE_RELU) o = fmaxf(o, 0.0f);
                    *cp = __float2bfloat16_rn(o);
                }
            }
        }
    }
}

// Persistent.  The scheduling unit is CL output tiles stacked along the rows: (row block pair (CL = 2)
// or row block, column block).  Cluster c (a single CTA when CL = 1) takes units c, c + clusters, ...;
// CTA `rank` of the cluster computes row block CL * pair + rank of each unit.  Warp 0 (lane 0) loads
// the operand tiles of every K block of those tiles into the stage ring; warp 1 (lane 0) issues the
// MMAs of tile j into TMEM accumulator j % 2 (2 x BN columns) and commits "acc full"; warps 2..5 read
// an accumulator (warp w reads TMEM lane quarter w % 4), store the tile and arrive on "acc empty", so
// the next tile's MMAs overlap this tile's stores.
//
// CL = 2: both CTAs of a unit need the same B tile.  Each producer loads its own A tile and one half
// of B, multicast into both CTAs at the same shared-memory offset, so a B tile leaves L2 once per
// pair (64 KB per K block and pair instead of 96 KB).  A stage is free for refilling once the MMAs
// of both CTAs have read it: every MMA issuer commits to the "empty" barrier of both CTAs (2 arrivals
// a phase).  Before a CTA exits, its producer waits until the peer's last commits have reached this
// CTA, then both producers exchange an arrival on a "done" barrier, so that no CTA leaves while the
// other still signals into its shared memory.  Rows past R (the second tile of a pair at an odd row
// block count) are zero-filled and never stored.
template <int BN, int CL>
__global__ void __launch_bounds__(192, 1) tc_rows_kernel(const __grid_constant__ TcParams p, const int total_units) {
    static_assert(CL == 1 || CL == 2, "clusters of 1 or 2 CTAs");
    constexpr uint32_t TC_TILE_B = tc_tile_b<BN>(), TC_STAGE = tc_stage<BN>(), TC_TMEM_COLS = 2 * BN;
    constexpr int TC_BN = BN;
    constexpr uint16_t PAIR = (uint16_t)((1u << CL) - 1u);  // both CTAs of the cluster
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t sbase = (raw + 1023u) & ~1023u;  // the swizzle atoms need 1024-byte alignment
    const uint32_t bars = sbase + TC_STAGES * TC_STAGE;
    const uint32_t full0 = bars, empty0 = bars + 8u * TC_STAGES;
    const uint32_t accf0 = bars + 16u * TC_STAGES, acce0 = accf0 + 16u;  // acc full / empty, 2 each
    const uint32_t tmem_slot = acce0 + 16u, done = tmem_slot + 8u;
    const uint32_t rank = CL > 1 ? tc_cluster_rank() : 0u;
    const int unit0 = CL > 1 ? (int)tc_cluster_id() : (int)blockIdx.x;
    const int ustep = CL > 1 ? (int)tc_cluster_count() : (int)gridDim.x;
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            tc_mbar_init(full0 + 8u * s, 1);
            tc_mbar_init(empty0 + 8u * s, CL);  // the MMA commits of every CTA of the cluster
        }
        for (int a = 0; a < 2; ++a) {
            tc_mbar_init(accf0 + 8u * a, 1);
            tc_mbar_init(acce0 + 8u * a, 4);  // the 4 epilogue warps
        }
        tc_mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tmem_slot),
                     "r"(TC_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    if constexpr (CL > 1) tc_cluster_sync();  // the peer's barriers exist before anything signals them
    else __syncthreads();
    tc_fence_after();
    uint32_t tmem;
    asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(tmem_slot) : "memory");
    // output tile of unit u of problem q for this CTA
    auto tile_of = [&](const TcProblem &q, int u, int &m0, int &n0) {
        const int local = u - q.tile_begin;
        m0 = ((local / q.tiles_n) * CL + (int)rank) * TC_BM;
        n0 = (local % q.tiles_n) * TC_BN;
    };

    if (warp == 0) {
        if (lane == 0) {
            // producer: operand tiles of every K block of every tile of this CTA
            int64_t g = 0;  // K blocks issued so far (stage g % STAGES)
            bool ok = true;
            for (int u = unit0; u < total_units && ok; u += ustep) {
                const TcProblem &q = p.prob[tc_problem_of(p, u)];
                int m0, n0;
                tile_of(q, u, m0, n0);
                for (int kb = 0; kb < q.kblocks; ++kb, ++g) {
                    const int s = (int)(g % TC_STAGES);
                    if (g >= TC_STAGES &&
                        !tc_wait(empty0 + 8u * s, (uint32_t)(((g / TC_STAGES) - 1) & 1), p.status, 21)) {
                        ok = false;
                        break;
                    }
                    const uint32_t st = sbase + (uint32_t)s * TC_STAGE;
                    tc_expect_tx(full0 + 8u * s, TC_STAGE);  // A, and all of B (half of it from the peer)
                    tc_tma_2d(st, &q.a_map, kb * TC_BK, m0, full0 + 8u * s);
                    if (q.b_mn) {
                        // B in place: BN / 64 copies of 64 columns x 64 K rows, 8 KB apart; this CTA's share
                        constexpr int PER = TC_BN / 64 / CL;
                        for (int jb = (int)rank * PER; jb < ((int)rank + 1) * PER; ++jb) {
                            const uint32_t dst = st + TC_TILE_A + 8192u * jb;
                            if constexpr (CL > 1)
                                tc_tma_2d_mc(dst, &q.b_map, n0 + 64 * jb, kb * TC_BK, full0 + 8u * s, PAIR);
                            else
                                tc_tma_2d(dst, &q.b_map, n0 + 64 * jb, kb * TC_BK, full0 + 8u * s);
                        }
                    } else if constexpr (CL > 1) {
                        // rows [rank * BN / 2, ...) of the K-major B tile (the map's box is BN / 2 rows)
                        tc_tma_2d_mc(st + TC_TILE_A + rank * (uint32_t)(TC_BN / 2) * 128u, &q.b_map, kb * TC_BK,
                                     n0 + (int)rank * (TC_BN / 2), full0 + 8u * s, PAIR);
                    } else {
                        tc_tma_2d(st + TC_TILE_A, &q.b_map, kb * TC_BK, n0, full0 + 8u * s);
                    }
                }
            }
            // before the CTA can finish, every copy issued has landed
            const int64_t tail = g - TC_STAGES > 0 ? g - TC_STAGES : 0;
            for (int64_t k = tail; k < g; ++k)
                tc_wait(full0 + 8u * (uint32_t)(k % TC_STAGES), (uint32_t)((k / TC_STAGES) & 1), p.status, 22);
            if constexpr (CL > 1) {
                // the peer's last commits have reached this CTA's empty barriers; then trade "done"
                for (int64_t k = tail; k < g; ++k)
                    tc_wait(empty0 + 8u * (uint32_t)(k % TC_STAGES), (uint32_t)((k / TC_STAGES) & 1), p.status, 26);
                tc_remote_arrive(done, rank ^ 1u);
                tc_wait_cluster(done, 0, p.status, 27);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN);
            int64_t g = 0;
            int j = 0;  // this CTA's tile count
            bool ok = true;
            for (int u = unit0; u < total_units && ok; u += ustep, ++j) {
                const TcProblem &q = p.prob[tc_problem_of(p, u)];
                const int a = j & 1;
                if (j >= 2 && !tc_wait(acce0 + 8u * a, (uint32_t)(((j >> 1) - 1) & 1), p.status, 25)) break;
                tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(a * TC_BN);
                for (int kb = 0; kb < q.kblocks; ++kb, ++g) {
                    const int s = (int)(g % TC_STAGES);
                    if (!tc_wait(full0 + 8u * s, (uint32_t)((g / TC_STAGES) & 1), p.status, 23)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t st = sbase + (uint32_t)s * TC_STAGE;
                    if (q.b_mn) {
                        // N-major B (transpose-B bit of the instruction descriptor); a 16-deep K step is
                        // 16 rows of 128 bytes
#pragma unroll
                        for (int k = 0; k < TC_BK / 16; ++k)
                            tc_mma(dacc, tc_desc(st + 32u * k), tc_desc_mn(st + TC_TILE_A + 2048u * k),
                                   idesc | (1u << 16), (kb | k) != 0);
                    } else {
#pragma unroll
                        for (int k = 0; k < TC_BK / 16; ++k)
                            tc_mma(dacc, tc_desc(st + 32u * k), tc_desc(st + TC_TILE_A + 32u * k), idesc,
                                   (kb | k) != 0);
                    }
                    // the stage is free once these MMAs (and the peer's) have read it
                    if constexpr (CL > 1) tc_commit_mc(empty0 + 8u * s, PAIR);
                    else tc_commit(empty0 + 8u * s);
                }
                tc_commit(accf0 + 8u * a);  // accumulator a holds tile j once these MMAs complete
            }
        }
    } else {
        // epilogue warps 2..5
        const int quarter = warp & 3;
        int j = 0;
        bool ok = true;
        for (int u = unit0; u < total_units; u += ustep, ++j) {
            const TcProblem &q = p.prob[tc_problem_of(p, u)];
            int m0, n0;
            tile_of(q, u, m0, n0);
            const int a = j & 1;
            ok = ok && __all_sync(0xffffffffu, tc_wait(accf0 + 8u * a, (uint32_t)((j >> 1) & 1), p.status, 24));
            tc_fence_after();
            if (!ok) break;
            tc_store_tile<BN>(q, m0, n0, quarter, lane, tmem + (uint32_t)(a * TC_BN), ok);  // adds the lane quarter
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

// BF16 matrix of `rows` x `cols` (row stride ld elements) as 64 x box_rows boxes with the 128-byte swizzle.
int tc_map(CUtensorMap *map, const void *base, int64_t cols, int64_t rows, int64_t ld, int box_rows) {
    auto enc = tc_encoder();
    SPREG_CHECK_ARG(enc, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SPREG_CHECK_ARG(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d) for a %lld x %lld BF16 operand", (int)r,
                    (long long)rows, (long long)cols);
    return SPREG_OK;
}

// Clusters of the tensor-core launches: 0 = automatic, 1 = single CTAs, 2 = CTA pairs sharing B.
std::atomic<int> g_tc_cluster{0};

cudaLaunchConfig_t tc_pair_config(cudaLaunchAttribute *attr, size_t smem, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(192);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// CTA pairs of tc_rows_kernel<BN, 2> that fit on device `dev` at once (a GPC's SMs may not all pair
// up; an SM-limited context may fit none): queried once per device, 0 when none fit.
template <int BN> int tc_max_pairs(int dev, int sms) {
    static std::atomic<int> max_pairs[64];  // per device: 0 = not queried, -1 = none fit
    if (dev < 0 || dev >= 64) return 0;
    int mc = max_pairs[dev].load();
    if (mc == 0) {
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = tc_pair_config(attr, tc_smem<BN>(), nullptr);
        cfg.gridDim = dim3((unsigned)(2 * (sms / 2 > 0 ? sms / 2 : 1)));
        if (cudaOccupancyMaxActiveClusters(&mc, tc_rows_kernel<BN, 2>, &cfg) != cudaSuccess || mc <= 0) {
            cudaGetLastError();  // a refused query leaves no error behind
            mc = -1;
        }
        max_pairs[dev].store(mc);
    }
    return mc > 0 ? mc : 0;
}

template <int BN, int CL>
cudaError_t tc_launch(const TcParams &p, int units, int sms, int pairs_fit, size_t smem, cudaStream_t stream) {
    if constexpr (CL == 1) {
        tc_rows_kernel<BN, 1><<<(unsigned)std::min(units, sms), 192, smem, stream>>>(p, units);
        return cudaGetLastError();
    } else {
        // as many clusters as fit at once, at most one per unit
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = tc_pair_config(attr, smem, stream);
        cfg.gridDim = dim3((unsigned)(2 * std::min(units, pairs_fit)));
        return cudaLaunchKernelEx(&cfg, tc_rows_kernel<BN, 2>, p, units);
    }
}

}  // namespace

void tc_set_cluster(int mode) { g_tc_cluster.store(mode); }

int dense_rows_batched_impl(const spreg_dense_rows_item *items, int32_t count, cudaStream_t stream) {
    SPREG_CHECK_ARG(count >= 0 && (count == 0 || items), "bad item list");
    int st = SPREG_OK;
    // checks; products with the same A, row index, output type and epilogue become one problem
    struct Group {
        const spreg_dense_rows_item *first;
        std::vector<int32_t> members;
        int64_t n = 0, bt_off = 0, tab_off = 0;
        bool mn = false;  // one product whose B is read in place (16-byte aligned rows): no transpose
    };
    std::vector<Group> groups;
    std::map<std::tuple<const void *, int64_t, int64_t, int64_t, const void *, int32_t, int32_t, int32_t>, size_t> key;
    for (int32_t i = 0; i < count; ++i) {
        const spreg_dense_rows_item &it = items[i];
        SPREG_CHECK_ARG(it.rows >= 0 && it.k >= 0 && it.n >= 0, "item %d: negative size", i);
        if (it.rows == 0 || it.n == 0) continue;
        SPREG_CHECK_ARG(it.a_rows && it.row_index && it.c && it.b, "item %d: null pointer", i);
        SPREG_CHECK_ARG(it.rows <= INT32_MAX && it.k <= INT32_MAX && it.n <= INT32_MAX, "item %d: size out of range", i);
        SPREG_CHECK_ARG(it.c_dtype == SPREG_F32 || it.c_dtype == SPREG_BF16, "item %d: C must be F32 or BF16", i);
        SPREG_CHECK_ARG(it.epilogue == SPREG_EPILOGUE_NONE || it.epilogue == SPREG_EPILOGUE_RELU, "item %d: bad epilogue",
                        i);
        SPREG_CHECK_ARG(it.lda >= it.k && (it.lda * 2) % 16 == 0 && reinterpret_cast<uintptr_t>(it.a_rows) % 16 == 0,
                        "A rows must be 16-byte aligned with a row stride of a multiple of 8 elements (item %d, lda "
                        "%lld)", i, (long long)it.lda);
        SPREG_CHECK_ARG(it.ldb >= it.n && it.ldc >= it.n, "item %d: ldb / ldc smaller than n", i);
        SPREG_CHECK_ARG(it.k > 0, "item %d: K must be positive", i);
        SPREG_CHECK_ARG(it.tile_n == 0 || it.tile_n == 128 || it.tile_n == 256, "item %d: tile_n must be 0, 128 or 256",
                        i);
        auto kk = std::make_tuple(it.a_rows, it.rows, it.k, it.lda, (const void *)it.row_index, it.c_dtype,
                                  it.load_c ? 1 : 0, it.epilogue);
        auto f = key.find(kk);
        if (f == key.end()) {
            key.emplace(kk, groups.size());
            groups.push_back(Group{&it, {i}, it.n});
        } else {
            Group &g = groups[f->second];
            g.members.push_back(i);
            g.n += it.n;
        }
    }
    if (groups.empty()) return SPREG_OK;
    // scratch: each transposed problem's Bt (n x K8, 256-byte aligned), then the segment tables
    int64_t bytes = 0;
    for (Group &g : groups) {
        SPREG_CHECK_ARG(g.n <= INT32_MAX, "coalesced products wider than 2^31 columns");
        const spreg_dense_rows_item &f = *g.first;
        g.mn = g.members.size() == 1 && reinterpret_cast<uintptr_t>(f.b) % 16 == 0 && (f.ldb * 2) % 16 == 0;
        if (g.mn) continue;
        const int64_t K8 = (f.k + 7) / 8 * 8;
        g.bt_off = bytes;
        bytes += (g.n * K8 * 2 + 255) / 256 * 256;
    }
    std::vector<unsigned char> tab;
    auto put = [&](const void *src, size_t len) {
        const size_t at = tab.size();
        tab.resize(at + (len + 7) / 8 * 8);
        memcpy(tab.data() + at, src, len);
        return (int64_t)at;
    };
    std::vector<int64_t> seg_c_off(groups.size(), 0), seg_ldc_off(groups.size(), 0);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        Group &g = groups[gi];
        if (g.members.size() < 2) continue;
        std::vector<int32_t> starts;
        std::vector<uint64_t> cs;
        std::vector<int64_t> lds;
        int32_t o = 0;
        for (int32_t m : g.members) {
            starts.push_back(o);
            o += (int32_t)items[m].n;
            cs.push_back(reinterpret_cast<uint64_t>(items[m].c));
            lds.push_back(items[m].ldc);
        }
        starts.push_back(o);
        g.tab_off = put(starts.data(), starts.size() * 4);
        seg_c_off[gi] = put(cs.data(), cs.size() * 8);
        seg_ldc_off[gi] = put(lds.data(), lds.size() * 8);
    }
    // transpose items (every member of every group), after the segment tables
    std::vector<TransposeItem> titems;
    int64_t max_kt = 1, max_nt = 1;
    for (Group &g : groups) {
        if (g.mn) continue;
        const int64_t K8 = (g.first->k + 7) / 8 * 8;
        int64_t o = 0;
        for (int32_t m : g.members) {
            const spreg_dense_rows_item &it = items[m];
            TransposeItem ti;
            ti.b = static_cast<const __nv_bfloat16 *>(it.b);
            ti.dst = nullptr;  // set once the scratch base is known
            ti.ldb = it.ldb;
            ti.k = (int32_t)it.k;
            ti.n = (int32_t)it.n;
            ti.K8 = (int32_t)K8;
            ti.pad = 0;
            titems.push_back(ti);
            max_kt = std::max<int64_t>(max_kt, (K8 + 63) / 64);
            max_nt = std::max<int64_t>(max_nt, (it.n + 63) / 64);
            o += it.n;
        }
    }
    SPREG_CHECK_ARG(titems.size() <= 65535 && max_nt <= 65535, "too many products in one call");
    const int64_t titem_off = put(titems.data(), titems.size() * sizeof(TransposeItem));  // dst filled in below
    const int64_t tab_base = (bytes + 255) / 256 * 256;
    int *status = device_status_word(&st);
    if (st != SPREG_OK) return st;
    static std::atomic<bool> configured[64];  // per device
    int dev = 0;
    SPREG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !configured[dev].load()) {
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<128, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<128>()));
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<256, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<256>()));
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<128, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<128>()));
        SPREG_CUDA(cudaFuncSetAttribute(tc_rows_kernel<256, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)tc_smem<256>()));
        configured[dev].store(true);
    }
    static std::atomic<int> sms_of[64];  // per device, 0 until queried
    if (dev >= 0 && dev < 64 && !sms_of[dev].load()) {
        int v = 0;
        SPREG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        sms_of[dev].store(v);
    }
    const int sms = (dev >= 0 && dev < 64 && sms_of[dev].load() > 0) ? sms_of[dev].load() : 148;
    char *scratch = nullptr;
    SPREG_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&scratch), (size_t)(tab_base + (int64_t)tab.size() + 16),
                               stream));
    auto fail = [&](int code) {
        cudaFreeAsync(scratch, stream);
        return code;
    };
    // B of every product, transposed into its problem's Bt at its segment's row offset: one launch
    {
        size_t t = 0;
        for (Group &g : groups) {
            if (g.mn) continue;
            const int64_t K8 = (g.first->k + 7) / 8 * 8;
            int64_t o = 0;
            for (int32_t m : g.members) {
                titems[t++].dst = reinterpret_cast<__nv_bfloat16 *>(scratch + g.bt_off) + o * K8;
                o += items[m].n;
            }
        }
    }
    memcpy(tab.data() + titem_off, titems.data(), titems.size() * sizeof(TransposeItem));
    cudaError_t e = cudaMemcpyAsync(scratch + tab_base, tab.data(), tab.size(), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && !titems.empty()) {
        transpose_items_kernel<<<dim3((unsigned)max_kt, (unsigned)max_nt, (unsigned)titems.size()), 256, 0,
                                 stream>>>(reinterpret_cast<const TransposeItem *>(scratch + tab_base + titem_off));
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        fail(0);
        SPREG_FAIL(SPREG_ERR_CUDA, "tensor-core set-up: %s", cudaGetErrorString(e));
    }
    static thread_local TcParams p;  // ~31 KB: kept off the stack
    for (size_t first = 0; first < groups.size(); first += TC_MAX_PROBLEMS) {
        const size_t cnt = std::min<size_t>(TC_MAX_PROBLEMS, groups.size() - first);
        memset(&p, 0, sizeof p);
        p.status = status;
        p.nprob = (int32_t)cnt;
        // 256-wide output tiles when every problem of the launch is wider than 128 columns, unless an
        // item asks for a width
        int64_t min_n = INT64_MAX;
        int hint = 0;
        for (size_t j = 0; j < cnt; ++j) {
            min_n = std::min<int64_t>(min_n, groups[first + j].n);
            for (int32_t m : groups[first + j].members)
                if (!hint && (items[m].tile_n == 128 || items[m].tile_n == 256)) hint = items[m].tile_n;
        }
        const int bn = hint ? hint : (min_n > 128 ? 256 : 128);
        // CTA pairs sharing B (cl = 2) when the launch has at least one full wave of pairs and the
        // padding of odd row block counts costs at most 1/8 of its tiles
        int64_t tiles1 = 0, pairs = 0;
        for (size_t j = 0; j < cnt; ++j) {
            const int64_t tm = (groups[first + j].first->rows + TC_BM - 1) / TC_BM;
            const int64_t tn = (groups[first + j].n + bn - 1) / bn;
            tiles1 += tm * tn;
            pairs += (tm + 1) / 2 * tn;
        }
        const int mode = g_tc_cluster.load();
        const int pairs_fit = mode == 1 ? 0 : bn == 256 ? tc_max_pairs<256>(dev, sms) : tc_max_pairs<128>(dev, sms);
        if (mode == 2 && pairs_fit == 0) {
            fail(0);
            SPREG_FAIL(SPREG_ERR_UNSUPPORTED, "tensor-core CTA pairs: no 2-CTA cluster fits this device or context");
        }
        const int cl = mode == 1 || pairs_fit == 0 ? 1
                       : mode == 2 ? 2
                                   : (pairs >= sms / 2 && 8 * (2 * pairs - tiles1) <= tiles1 ? 2 : 1);
        int64_t tiles = 0;
        for (size_t j = 0; j < cnt; ++j) {
            const size_t gi = first + j;
            const Group &g = groups[gi];
            const spreg_dense_rows_item &it = *g.first;
            TcProblem &q = p.prob[j];
            const int64_t K8 = (it.k + 7) / 8 * 8;
            q.row_index = it.row_index;
            q.C = it.c;
            q.ldc = it.ldc;
            q.R = (int32_t)it.rows;
            q.n = (int32_t)g.n;
            q.kblocks = (int32_t)((it.k + TC_BK - 1) / TC_BK);
            q.c_dtype = it.c_dtype;
            q.load_c = it.load_c ? 1 : 0;
            q.epilogue = it.epilogue;
            q.nseg = (int32_t)g.members.size();
            if (q.nseg > 1) {
                q.seg_start = reinterpret_cast<const int32_t *>(scratch + tab_base + g.tab_off);
                q.seg_c = reinterpret_cast<void *const *>(scratch + tab_base + seg_c_off[gi]);
                q.seg_ldc = reinterpret_cast<const int64_t *>(scratch + tab_base + seg_ldc_off[gi]);
            }
            q.tiles_n = (int32_t)((g.n + bn - 1) / bn);
            q.tile_begin = (int32_t)tiles;  // in units of cl row blocks x one column block
            tiles += ((it.rows + TC_BM - 1) / TC_BM + cl - 1) / cl * q.tiles_n;
            q.b_mn = g.mn ? 1 : 0;
            if ((st = tc_map(&q.a_map, it.a_rows, it.k, it.rows, it.lda, TC_BM)) ||
                (st = g.mn ? tc_map(&q.b_map, it.b, g.n, it.k, it.ldb, 64)
                           : tc_map(&q.b_map, scratch + g.bt_off, it.k, g.n, K8, bn / cl)))
                return fail(st);
        }
        if (tiles > INT32_MAX) {
            fail(0);
            SPREG_FAIL(SPREG_ERR_UNSUPPORTED, "too many output tiles in one launch");
        }
        if (bn == 256) e = cl == 2 ? tc_launch<256, 2>(p, (int)tiles, sms, pairs_fit, tc_smem<256>(), stream)
                                   : tc_launch<256, 1>(p, (int)tiles, sms, pairs_fit, tc_smem<256>(), stream);
        else e = cl == 2 ? tc_launch<128, 2>(p, (int)tiles, sms, pairs_fit, tc_smem<128>(), stream)
                         : tc_launch<128, 1>(p, (int)tiles, sms, pairs_fit, tc_smem<128>(), stream);
        if (e != cudaSuccess) {
            fail(0);
            SPREG_FAIL(SPREG_ERR_CUDA, "tensor-core launch: %s", cudaGetErrorString(e));
        }
    }
    cudaFreeAsync(scratch, stream);
    return SPREG_OK;
}

int dense_rows_bf16_impl(const void *a_rows, int64_t R, int64_t K, int64_t lda, const int32_t *row_index,
                         const void *b, int64_t ldb, void *c, int64_t ldc, int64_t n, int32_t c_dtype, int32_t load_c,
                         int32_t epilogue, cudaStream_t stream) {
    const spreg_dense_rows_item it = {a_rows, R, K, lda, row_index, b, ldb, c, ldc, n, c_dtype, load_c, epilogue, 0};
    return dense_rows_batched_impl(&it, 1, stream);
}

}  // namespace spreg
