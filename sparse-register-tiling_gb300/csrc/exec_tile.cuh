// exec_tile.cuh -- executor variant that stages B in shared memory, one K tile at a time.
//
// A job is (problem, group of W row panels, strip of 32 * NV columns).  One CTA runs W consumer
// warps (warp w owns panel group * W + w, its accumulators in registers as in exec_batch_kernel)
// and one producer warp.  For every K tile t of the job the producer copies
//   * the tile's B rows [col_offset + t * K_c, ... + K_c) x the strip's columns: one 2-D tensor
//     copy (TMA, a tensor map of B per problem) per 256 rows, zero-filled outside B, and
//   * the execution blocks of units (panel, t) of all consumer warps: one bulk copy when the
//     blocks are adjacent in memory (panels of one row tile), else one per warp
// into one stage of a ring of kTileStages stages, and arrives on the stage's "full" barrier
// (expect_tx of all bytes).  Consumers gather B rows out of shared memory (one broadcast-free
// 4 * NV-byte load per lane per entry) and arrive on the stage's "empty" barrier when done; the
// producer refills a stage after all W consumers released it.  Jobs follow each other through
// the same ring, so the producer fetches the next job's first tile while consumers finish the
// last tile of the current one.
//
// The W panels of a job are consecutive in the pack's work order (panels by descending work), so
// a job's warps finish each K tile at about the same time and the stage is refilled without a
// long wait on the slowest warp; their execution blocks of one K tile are adjacent in memory.
//
// B rows are read from L2 once per job instead of once per packed entry: for the W panels of a
// job a B row is copied once, while the gathers of exec_batch_kernel fetch it once per entry
// that references it (about W * (1 - sparsity^M_r) times).  Per output element the FMA chain is
// the same as the other executors (K tiles in order, entries in packed order), so the results
// are bit-identical.
//
// Panel rounds (TileParams::rounds > 1, any K tiling): a job is R rounds of W panels on one strip.
// The strip of B for every K tile stays in shared memory for the whole job (one of nbuf resident
// buffers, loaded by the job's first stage), and the ring stages carry only the execution blocks
// of one round's units (round r, K tile t).  A B row then comes from L2 once per W * R panels:
// at high sparsity, where a job of W panels gathers about as many B bytes as its stage copies,
// this divides the L2-to-SM traffic by R.  The FMA chain per element is unchanged.
//
// Every wait is bounded; a wait that gives up records a code in the device status word and the
// warp stops, the producer first waiting (bounded) for the copies it issued.
#pragma once
#include <atomic>
#include <cuda.h>

#include <cstddef>
#include <type_traits>

#include "exec_kernel.cuh"

namespace spreg {

constexpr int kTileStages = 2;      // ring stages of a launch without panel rounds
constexpr int kTileMaxStages = 4;   // ring stages with panel rounds (metadata only, small)
constexpr int kTileMaxRounds = 64;  // panel rounds per job
constexpr int kTileMaxWarps = 15;   // consumer warps per CTA (with the producer: 512 threads, 128 registers each)
constexpr int kTileMaxProblems = 96; // problems per launch (a tensor map each; kernel parameters <= 32 KB)
constexpr int kTileBoxRows = 256;    // rows of one tensor copy (TMA box limit)

struct TProblem {
    const uint8_t *exec;        // execution layout of the packed matrix
    const int64_t *exec_offs;   // units + 1 block offsets in slot order (exec_slot)
    const int32_t *panel_order; // panels by descending work: job group g runs panel_order[g * W + w] on warp w
    const float *scales;        // per-row-panel F16 scales (else null)
    const void *B;
    void *C;
    int64_t ldb, ldc;
    int32_t M;                  // rows of A and C
    int32_t job_begin;          // first global job
    int32_t col_begin;          // first column of the problem's strips
    int32_t col_end;            // columns >= col_end are not computed
    int32_t P, S, T;            // row panels (work-order positions), strips, K tiles
    int16_t combine;            // load-balanced halves: 0 none, 1 low half (flags its stores), 2 high half
                                // (waits for the low half, then C = C + acc)
    int16_t pad16;
    int16_t load_c, epilogue;
    int16_t order;              // job order: 0 = panel groups outer (a group's strips in a row), 1 = strips outer
    int16_t box_rows;           // rows of one tensor copy (K tile copied in ceil(kt / box_rows) copies)
    int32_t kt;                 // B rows per K tile
    int32_t flag_off;           // combine: flags of (position - pos_begin, strip) at flags[flag_off + pos * S + strip]
    int32_t col_offset;         // first B row of tile 0
    // The units this problem runs: K tiles [t_begin, t_end) of the panels at work-order positions
    // [pos_begin, pos_begin + count) (the whole pack: 0, T, 0, P).  A load-balanced SpMM splits its
    // heaviest panels' K tiles between two problems (spreg_exec_args.load_balance).
    int16_t t_begin, t_end;
    int32_t pos_begin, count;
    CUtensorMap tmap;           // B as a 2-D tensor: columns [0, col_end) x rows [0, col_offset + krows)
};
static_assert(sizeof(TProblem) == 256 && offsetof(TProblem, tmap) == 128, "TProblem layout");

struct TileParams {
    int *counter;               // job counter, zero at launch
    int *status;                // device status word of bounded waits
    int64_t jobs;               // total jobs
    int32_t nprob;
    int32_t xbuf;               // bytes of one consumer's metadata slot
    int32_t warps;              // consumer warps W
    int32_t stage_b;            // bytes of one stage's B tile; with panel rounds, of one resident B strip
    int32_t stages;             // ring stages (2 .. kTileMaxStages)
    int32_t rounds;             // panel rounds per job (1: B tiles travel in the ring stages)
    int32_t nbuf;               // resident B strips (1 or 2) with panel rounds, else 0
    int32_t pad_;
    int *flags;                 // load-balance flags (zero at launch), indexed by TProblem::flag_off
    TProblem prob[kTileMaxProblems];
};
static_assert(sizeof(TileParams) <= 32764, "kernel parameters are limited to 32764 bytes");

__device__ __forceinline__ int find_tproblem(const TileParams &tp, int64_t job) {
    int lo = 0, hi = tp.nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tp.prob[mid].job_begin <= job) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One box of a 2-D tensor map (columns x, rows y) into shared memory; rows and columns outside
// the tensor read as zero.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void sts_u32(uint32_t a, uint32_t v) {
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void sts_v4(uint32_t a, int x, int y, int z, int w) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(x), "r"(y), "r"(z), "r"(w) : "memory");
}
__device__ __forceinline__ int4 lds_v4(uint32_t a) {
    int4 v;
    asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a)
                 : "memory");
    return v;
}

// B rows of one lane's columns out of a shared-memory tile: row c of B is tile row c - r0.
template <int NV, class TB> struct SmemB {
    uint32_t base;       // tile + this lane's first column - r0 * row_bytes (mod 2^32): B row c is at
                         // base + c * row_bytes, one shift-add per entry
    uint32_t row_bytes;  // 32 * NV * sizeof(TB)
    // 16-bit B, NV = 8: the lane's 8 columns as 4 packed words (for the mixed-precision FMA)
    __device__ __forceinline__ void load_raw(int k, uint32_t (&w)[NV / 2]) const {
        static_assert(sizeof(TB) == 2 && NV == 8, "packed B rows are 16-bit, 8 columns per lane");
        const uint4 v = lds_u128(base + (uint32_t)k * row_bytes);
        w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
    }
    __device__ __forceinline__ void load(int k, float (&b)[NV]) const {
        const uint32_t a = base + (uint32_t)k * row_bytes;
        if constexpr (sizeof(TB) == 4) {
            if constexpr (NV == 1) {
                b[0] = __uint_as_float(lds_u32(a));
            } else if constexpr (NV == 2) {
                const uint2 v = lds_u64(a);
                b[0] = __uint_as_float(v.x); b[1] = __uint_as_float(v.y);
            } else {
#pragma unroll
                for (int i = 0; i < NV / 4; ++i) {
                    const uint4 v = lds_u128(a + 16u * i);
                    b[4 * i] = __uint_as_float(v.x); b[4 * i + 1] = __uint_as_float(v.y);
                    b[4 * i + 2] = __uint_as_float(v.z); b[4 * i + 3] = __uint_as_float(v.w);
                }
            }
        } else {
            if constexpr (NV == 1) {
                b[0] = word_val<TB>(lds_u16(a), 0);
            } else if constexpr (NV == 2) {
                const uint32_t w = lds_u32(a);
                b[0] = word_val<TB>(w, 0); b[1] = word_val<TB>(w, 1);
            } else if constexpr (NV == 4) {
                const uint2 v = lds_u64(a);
                b[0] = word_val<TB>(v.x, 0); b[1] = word_val<TB>(v.x, 1);
                b[2] = word_val<TB>(v.y, 0); b[3] = word_val<TB>(v.y, 1);
            } else {
                const uint4 v = lds_u128(a);
                b[0] = word_val<TB>(v.x, 0); b[1] = word_val<TB>(v.x, 1);
                b[2] = word_val<TB>(v.y, 0); b[3] = word_val<TB>(v.y, 1);
                b[4] = word_val<TB>(v.z, 0); b[5] = word_val<TB>(v.z, 1);
                b[6] = word_val<TB>(v.w, 0); b[7] = word_val<TB>(v.w, 1);
            }
        }
    }
    __device__ __forceinline__ void load(int k, BSeg<NV, TB> &b) const {
        if constexpr (sizeof(TB) == 4) {
            load(k, b.f);
        } else {
            const uint32_t a = base + (uint32_t)k * row_bytes;
            if constexpr (NV == 1) {
                b.w[0] = (uint32_t)lds_u16(a);
            } else if constexpr (NV == 2) {
                b.w[0] = lds_u32(a);
            } else if constexpr (NV == 4) {
                const uint2 v = lds_u64(a);
                b.w[0] = v.x; b.w[1] = v.y;
            } else {
                load_raw(k, b.w);
            }
        }
    }
};

// C tile init / store of one (problem, panel, strip), as x_acc_init / x_store.
template <int MR, int NV, class TV, class TC>
__device__ __forceinline__ void t_acc_init(const TProblem &pr, int64_t row0, int64_t col0, bool valid,
                                           float (&acc)[MR][NV]) {
    constexpr bool SCALED = std::is_same<TV, __half>::value;
#pragma unroll
    for (int r = 0; r < MR; ++r)
#pragma unroll
        for (int j = 0; j < NV; ++j) acc[r][j] = 0.0f;
    if (!SCALED && pr.load_c && valid) {
        const TC *C = reinterpret_cast<const TC *>(pr.C);
#pragma unroll
        for (int r = 0; r < MR; ++r)
            if (row0 + r < pr.M) VecIO<NV, TC>::load_plain(C + (row0 + r) * pr.ldc + col0, acc[r]);
    }
}
template <int MR, int NV, class TV, class TC>
__device__ __forceinline__ void t_store(const TProblem &pr, int64_t gp, int64_t row0, int64_t col0, bool valid,
                                        const float (&acc)[MR][NV]) {
    if (!valid) return;
    constexpr bool SCALED = std::is_same<TV, __half>::value;
    TC *C = reinterpret_cast<TC *>(pr.C);
    const float s = SCALED ? pr.scales[gp] : 1.0f;
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        if (row0 + r >= pr.M) continue;
        TC *cp = C + (row0 + r) * pr.ldc + col0;
        float o[NV];
#pragma unroll
        for (int j = 0; j < NV; ++j) o[j] = acc[r][j];
        if (SCALED) {
            if (pr.load_c) {
                float cin[NV];
                VecIO<NV, TC>::load_plain(cp, cin);
#pragma unroll
                for (int j = 0; j < NV; ++j) o[j] = fmaf(o[j], s, cin[j]);
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) o[j] = o[j] * s;
            }
        }
        if (pr.epilogue == SPREG_EPILOGUE_RELU) {
#pragma unroll
            for (int j = 0; j < NV; ++j) o[j] = fmaxf(o[j], 0.0f);
        }
        VecIO<NV, TC>::store(cp, o);
    }
}

// High half of a load-balanced (panel, strip): C = C + acc (one FP32 add per element, the low half's
// stored result first), then the epilogue.  The low half's stores are visible: every lane acquired
// the flag its warp released after them.
template <int MR, int NV, class TV, class TC>
__device__ __forceinline__ void t_store_add(const TProblem &pr, int64_t row0, int64_t col0, bool valid,
                                            const float (&acc)[MR][NV]) {
    if (!valid) return;
    TC *C = reinterpret_cast<TC *>(pr.C);
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        if (row0 + r >= pr.M) continue;
        TC *cp = C + (row0 + r) * pr.ldc + col0;
        float o[NV];
        VecIO<NV, TC>::load_plain(cp, o);
#pragma unroll
        for (int j = 0; j < NV; ++j) o[j] = o[j] + acc[r][j];
        if (pr.epilogue == SPREG_EPILOGUE_RELU) {
#pragma unroll
            for (int j = 0; j < NV; ++j) o[j] = fmaxf(o[j], 0.0f);
        }
        VecIO<NV, TC>::store(cp, o);
    }
}

// Bounded wait for a load-balance flag (acquire, GPU scope).  Gives up after about a second,
// recording `code` in the device status word.
__device__ __forceinline__ bool lb_flag_wait(const int *f, int *status, int code) {
    for (uint32_t it = 0; it < (1u << 23); ++it) {
        int v;
        asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
        if (v) return true;
        if (it >= 32) __nanosleep(128);
    }
    atomicCAS(status, 0, code);
    return false;
}
__device__ __forceinline__ void lb_flag_release(int *f) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(f), "r"(1) : "memory");
}

// Shared memory: [0, 64) full / empty barriers, [256, 256 + 16 * stages) job of each stage,
// [512, 512 + 4 * 16 * stages) each consumer's block offset in each stage's metadata area, from
// 1024 the stages: B tile (stage_b bytes) then the metadata area (W * xbuf bytes).
// GEN: the general form (panel rounds, per-problem K-tile and work-order ranges, load-balanced
// halves); without it the launch runs whole problems through a ring of kTileStages stages with those
// checks compiled out (the plain executor's hot path).
template <int MR, int NV, class TV, class TB, class TC, bool GEN>
__global__ void __launch_bounds__(32 * (kTileMaxWarps + 1), 1) exec_tile_kernel(const __grid_constant__ TileParams tp) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr uint32_t ROWB = 32u * NV * (uint32_t)sizeof(TB);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = tp.warps;
    const int NS = GEN ? tp.stages : kTileStages;
    const int R = GEN ? tp.rounds : 1;
    const bool res = GEN && tp.nbuf > 0;  // panel rounds: B strips resident outside the ring
    // a problem's K tiles [t_begin, t_end) and work-order positions [pos_begin, pos_begin + count)
    auto t_lo = [](const TProblem &pr) -> int { return GEN ? (int)pr.t_begin : 0; };
    auto t_hi = [](const TProblem &pr) -> int { return GEN ? (int)pr.t_end : pr.T; };
    auto p_lo = [](const TProblem &pr) -> int64_t { return GEN ? (int64_t)pr.pos_begin : 0; };
    auto p_n = [](const TProblem &pr) -> int64_t { return GEN ? (int64_t)pr.count : (int64_t)pr.P; };
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t full0 = sbase, empty0 = sbase + 8u * kTileMaxStages, jobs0 = sbase + 256u, moffs0 = sbase + 512u;
    const uint32_t res0 = sbase + 1024u;                          // resident B strips (panel rounds)
    const uint32_t meta_off = res ? 0u : (uint32_t)tp.stage_b;    // execution blocks within a ring stage
    const uint32_t stage_bytes = meta_off + (uint32_t)W * (uint32_t)tp.xbuf;
    const uint32_t stage0 = res0 + (res ? (uint32_t)tp.nbuf * (uint32_t)tp.stage_b : 0u);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(full0 + 8u * s, 1);
            mbar_init(empty0 + 8u * s, (uint32_t)W);
        }
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();

    if (warp == W) {
        // ------------------------------------------------------------ producer
        int pi = -1, group = 0, strip = 0, t = 0, r = 0, rounds_job = 1;
        int64_t njob = 0;  // jobs fetched by this CTA: job j reads resident strip j % nbuf
        auto fetch = [&]() {
            int it = 0;
            if (lane == 0) it = atomicAdd(tp.counter, 1);
            const int64_t job = __shfl_sync(0xffffffffu, it, 0);
            if (job >= tp.jobs) {
                pi = -1;
                return;
            }
            pi = find_tproblem(tp, job);
            const TProblem &pr = tp.prob[pi];
            const int64_t local = job - pr.job_begin;
            const int64_t gsz = (int64_t)W * R;  // panels per job
            if (pr.order == 1) {
                const int64_t groups = (p_n(pr) + gsz - 1) / gsz;
                group = (int)(local % groups);
                strip = (int)(local / groups);
            } else {
                group = (int)(local / pr.S);
                strip = (int)(local % pr.S);
            }
            t = t_lo(pr);
            r = 0;
            const int64_t left = p_n(pr) - (int64_t)group * gsz;  // panels from this job's first on
            rounds_job = (int)((left + W - 1) / W < R ? (left + W - 1) / W : R);
            ++njob;
        };
        fetch();
        // ring position: fill `seq` goes to stage s in fill round rnd (seq = rnd * NS + s), kept
        // incrementally (no division per stage)
        uint32_t last_rnd[kTileMaxStages];  // fill round of each stage's last fill
        bool filled[kTileMaxStages];
#pragma unroll
        for (int i = 0; i < kTileMaxStages; ++i) {
            last_rnd[i] = 0;
            filled[i] = false;
        }
        // the last stage that read each resident strip: its fill number, stage and round
        int64_t buf_last[2] = {-1, -1};
        int buf_stage[2] = {0, 0};
        uint32_t buf_rnd[2] = {0, 0};
        bool ok = true;
        int s = 0;
        uint32_t rnd = 0;
#pragma unroll 1
        for (int64_t seq = 0;; ++seq) {
            const uint32_t full = full0 + 8u * s, empty = empty0 + 8u * s;
            if (rnd > 0 && !mbar_wait_bounded(empty, (rnd - 1) & 1u, tp.status, 5)) {
                ok = false;
                break;
            }
            if (pi < 0) {
                if (lane == 0) {
                    sts_v4(jobs0 + 16u * s, -1, 0, 0, 0);
                    mbar_arrive(full);
                }
                break;
            }
            const TProblem &pr = tp.prob[pi];
            const int c0 = pr.col_begin + strip * (32 * NV);
            const int nbox = (pr.kt + pr.box_rows - 1) / pr.box_rows;
            const int b = res ? (int)((njob - 1) & (int64_t)(tp.nbuf - 1)) : 0;  // nbuf is 1 or 2
            const bool load_b = !res || (r == 0 && t == t_lo(pr));
            if (res && load_b) {
                // the job that read this strip before must be done with it: its last stage released
                // (a stage NS or more back is already covered by the ring wait above)
                const int64_t L = buf_last[b];
                if (L >= 0 && seq - L < NS &&
                    !mbar_wait_bounded(empty0 + 8u * (uint32_t)buf_stage[b], buf_rnd[b] & 1u, tp.status, 8)) {
                    ok = false;
                    break;
                }
            }
            // metadata: lane w < W holds the block of unit (panel pos_begin + (group * R + r) * W + w, t)
            int64_t moff = 0;
            uint32_t mbytes = 0;
            const int64_t pos = p_lo(pr) + ((int64_t)group * R + r) * W + lane;  // position in the work order
            const bool act = lane < W && pos < p_lo(pr) + p_n(pr);
            if (act) {
                const int64_t slot = (int64_t)t * pr.P + pos;
                moff = pr.exec_offs[slot];
                mbytes = (uint32_t)(pr.exec_offs[slot + 1] - moff);
            }
            const int nact = __popc(__ballot_sync(0xffffffffu, act));  // active lanes are 0 .. nact - 1
            const int64_t m0 = __shfl_sync(0xffffffffu, moff, 0);
            const int64_t nxt = __shfl_down_sync(0xffffffffu, moff, 1);
            const bool contig = __all_sync(0xffffffffu, !(act && lane + 1 < nact) || moff + mbytes == nxt);
            uint32_t mtotal = mbytes;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mtotal += __shfl_xor_sync(0xffffffffu, mtotal, o);
            if (lane < W)
                sts_u32(moffs0 + 4u * (uint32_t)(s * kTileMaxWarps + lane),
                        contig ? (uint32_t)(moff - m0) : (uint32_t)lane * (uint32_t)tp.xbuf);
            const uint32_t sb = stage0 + (uint32_t)s * stage_bytes;
            const uint32_t tile_b = (uint32_t)(nbox * pr.box_rows) * ROWB;  // one K tile of the strip
            if (lane == 0) {
                sts_v4(jobs0 + 16u * s, pi, group * R + r, strip, t | (b << 16));
                const uint32_t bbytes = load_b ? (res ? (uint32_t)(t_hi(pr) - t_lo(pr)) : 1u) * tile_b : 0u;
                mbar_arrive_expect_tx(full, bbytes + mtotal);
                if (res && load_b) {
                    // every K tile of the problem's range, into resident strip b (tile tt at tt * tile_b)
                    const uint32_t dst = res0 + (uint32_t)b * (uint32_t)tp.stage_b;
                    for (int tt = t_lo(pr); tt < t_hi(pr); ++tt)
                        for (int bx = 0; bx < nbox; ++bx)
                            tma_load_2d(dst + (uint32_t)tt * tile_b + (uint32_t)(bx * pr.box_rows) * ROWB, &pr.tmap, c0,
                                        pr.col_offset + tt * pr.kt + bx * pr.box_rows, full);
                } else if (load_b) {
                    const int r0 = pr.col_offset + t * pr.kt;
                    for (int bx = 0; bx < nbox; ++bx)
                        tma_load_2d(sb + (uint32_t)(bx * pr.box_rows) * ROWB, &pr.tmap, c0, r0 + bx * pr.box_rows,
                                    full);
                }
                if (contig && mtotal) bulk_copy_g2s(sb + meta_off, pr.exec + m0, mtotal, full);
            }
            if (!contig && mbytes)
                bulk_copy_g2s(sb + meta_off + (uint32_t)lane * (uint32_t)tp.xbuf, pr.exec + moff, mbytes, full);
            __syncwarp();
            filled[s] = true;
            last_rnd[s] = rnd;
            if (res) {
                buf_last[b] = seq;
                buf_stage[b] = s;
                buf_rnd[b] = rnd;
            }
            if (++t == t_hi(pr)) {
                t = t_lo(pr);
                if (++r == rounds_job) fetch();
            }
            if (++s == NS) {
                s = 0;
                ++rnd;
            }
        }
        if (!ok) {
            // copies still in flight land in stages whose full barrier has not flipped yet
            for (int i = 0; i < NS; ++i)
                if (filled[i]) mbar_wait_bounded(full0 + 8u * i, last_rnd[i] & 1u, tp.status, 7);
        }
        return;
    }

    // ---------------------------------------------------------------- consumers
    float acc[MR][NV];
    int s = 0;          // stage of this fill
    uint32_t rnd = 0;   // its fill round (the full barrier's phase parity)
#pragma unroll 1
    for (;;) {
        if (!mbar_wait_bounded(full0 + 8u * s, rnd & 1u, tp.status, 6)) break;
        const int4 ji = lds_v4(jobs0 + 16u * s);
        if (ji.x < 0) break;
        const TProblem &pr = tp.prob[ji.x];
        const int64_t pos = p_lo(pr) + (int64_t)ji.y * W + warp;
        const int t = ji.w & 0xffff;
        if (pos < p_lo(pr) + p_n(pr)) {
            const int64_t gp = pr.panel_order[pos];
            const int64_t row0 = gp * MR;
            const int64_t col0 = pr.col_begin + (int64_t)ji.z * (32 * NV) + (int64_t)lane * NV;
            const bool valid = col0 < pr.col_end;
            if (t == t_lo(pr)) t_acc_init<MR, NV, TV, TC>(pr, row0, col0, valid, acc);
            const uint32_t sb = stage0 + (uint32_t)s * stage_bytes;
            // B tile t: in the ring stage, or in resident strip ji.w >> 16
            uint32_t bt = sb;
            if (res) {
                const uint32_t tile_b = (uint32_t)((pr.kt + pr.box_rows - 1) / pr.box_rows * pr.box_rows) * ROWB;
                bt = res0 + (uint32_t)(ji.w >> 16) * (uint32_t)tp.stage_b + (uint32_t)t * tile_b;
            }
            const uint32_t buf = sb + meta_off + lds_u32(moffs0 + 4u * (uint32_t)(s * kTileMaxWarps + warp));
            const uint32_t r0 = (uint32_t)(pr.col_offset + t * pr.kt);  // B row of tile row 0
            const SmemB<NV, TB> bl{bt + (uint32_t)lane * (uint32_t)(NV * sizeof(TB)) - r0 * ROWB, ROWB};
            const uint32_t G = lds_u32(buf);
#pragma unroll 1
            for (uint32_t g = 0; g < G; ++g) {
                const uint4 rec = lds_u128(buf + 16u + 16u * g);
                run_group_x<MR, NV, TV, true>((int)rec.x, (int)rec.y, buf + rec.z, buf + rec.w, bl, acc);
            }
            if (t == t_hi(pr) - 1) {
                if (!GEN || pr.combine == 0) {
                    t_store<MR, NV, TV, TC>(pr, gp, row0, col0, valid, acc);
                } else {
                    int *fl = tp.flags + pr.flag_off + (pos - pr.pos_begin) * pr.S + ji.z;
                    if (pr.combine == 1) {
                        // low half: store, then release this (panel, strip)'s flag
                        t_store<MR, NV, TV, TC>(pr, gp, row0, col0, valid, acc);
                        __threadfence();
                        __syncwarp();
                        if (lane == 0) lb_flag_release(fl);
                    } else if (lb_flag_wait(fl, tp.status, 9)) {
                        // high half: after the low half's stores, C = C + acc
                        t_store_add<MR, NV, TV, TC>(pr, row0, col0, valid, acc);
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8u * s);
        if (++s == NS) {
            s = 0;
            ++rnd;
        }
    }
}

// 256-column strips (NV = 8) are built for 16-bit B and M_r <= 4 only.
using TileKernelPtr = void (*)(TileParams);
template <int MR, class V, class B, class C, bool GEN> inline TileKernelPtr tile_nv8_kernel() {
    if constexpr (sizeof(B) == 2 && MR <= 4) return exec_tile_kernel<MR, 8, V, B, C, GEN>;
    else return nullptr;
}

template <int MR, int COMBO>
cudaError_t launch_exec_tile(const TileParams &p, int nv, bool gen, unsigned grid, int threads, size_t smem,
                             cudaStream_t s);

#define SPREG_INSTANTIATE_TILE(MR, COMBO)                                                             \
    template <>                                                                                       \
    cudaError_t launch_exec_tile<MR, COMBO>(const TileParams &p, int nv, bool gen, unsigned grid, int threads, \
                                            size_t smem, cudaStream_t s) {                            \
        using V = ComboTypes<COMBO>::V;                                                               \
        using B = ComboTypes<COMBO>::B;                                                               \
        using C = ComboTypes<COMBO>::C;                                                               \
        static std::atomic<bool> configured[64][9][2];                                                \
        int dev = 0;                                                                                  \
        cudaGetDevice(&dev);                                                                          \
        auto run = [&](auto kern) -> cudaError_t {                                                    \
            if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;                                  \
            if (!configured[dev][nv][gen].load()) {                                                   \
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem); \
                if (e != cudaSuccess) return e;                                                       \
                configured[dev][nv][gen].store(true);                                                 \
            }                                                                                         \
            /* at most the CTAs that can be resident at once (registers included) */                  \
            int occ = 0, nsm = 0;                                                                     \
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem) == cudaSuccess && occ > 0 && \
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && nsm > 0) \
                grid = std::min<unsigned>(grid, (unsigned)occ * (unsigned)nsm);                       \
            kern<<<grid, threads, smem, s>>>(p);                                                      \
            return cudaGetLastError();                                                                \
        };                                                                                            \
        auto pick = [&](auto gtag) -> cudaError_t {                                                   \
            constexpr bool G = decltype(gtag)::value;                                                 \
            switch (nv) {                                                                             \
            case 1: return run(exec_tile_kernel<MR, 1, V, B, C, G>);                                  \
            case 2: return run(exec_tile_kernel<MR, 2, V, B, C, G>);                                  \
            case 4: return run(exec_tile_kernel<MR, 4, V, B, C, G>);                                  \
            case 8: {                                                                                 \
                auto k8 = tile_nv8_kernel<MR, V, B, C, G>();                                          \
                return k8 ? run(k8) : cudaErrorInvalidValue;                                          \
            }                                                                                         \
            default: return cudaErrorInvalidValue;                                                    \
            }                                                                                         \
        };                                                                                            \
        return gen ? pick(std::true_type{}) : pick(std::false_type{});                                \
    }

}  // namespace spreg
