// exec_kernel.cuh -- the sparse-register-tiling executor for sm_103a.
//
// Semantics (sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305 and
// tools/codegen/gen_vector_specialized.py:266-357): for a row panel of M_r rows and a strip of
// columns, the M_r x strip accumulator tile starts at C (load_c) or zero; for every nanokernel
// id in order and for nkern_counts[id] entries, the B row named by the entry's column index is
// multiplied by the entry's values, one per set row of the id's pattern in ascending row order.
//
// GPU mapping: one warp owns one row panel x (32 * NV) columns; lane l keeps NV consecutive
// columns of every panel row in registers (acc[MR][NV]).  nkern_counts make the per-id loops
// warp-uniform, and the switch below gives every pattern its own loop with compile-time register
// indices -- the role the reference's generated nanokernels play.  Each output element is an
// fmaf chain in packed-entry order, identical to the CPU executor's.
#pragma once
#include <atomic>

#include <type_traits>

#include "spreg_common.cuh"

namespace spreg {

struct ExecParams {
    const uint8_t *arena;
    const spreg_panel_desc *descs;
    const float *scales;
    const void *B;
    void *C;
    int64_t ldb, ldc, M, N;
    int64_t col_begin;  // first column handled by this launch
    int64_t P, ppt, T;
    int64_t b_row0, b_rows;  // rows of B the packed column indices reach (staged kernel)
    int *status;             // device status word: set when a bounded wait gives up
    const uint8_t *exec;     // execution layout blocks (one per unit)
    const int64_t *exec_offs;
    int32_t xbuf;            // bytes of one per-warp metadata buffer (>= largest block)
    int32_t pad2_;
    int32_t nk, load_c, epilogue, pad_;
    uint8_t id_pattern[256];
};

__host__ __device__ constexpr int cpopc(int x) { return x == 0 ? 0 : (x & 1) + cpopc(x >> 1); }

// ------------------------------------------------------------------ vector loads / stores
template <int NV, class T> struct VecIO;

template <int NV> struct VecIO<NV, float> {
    __device__ static void load(const float *__restrict__ p, float (&b)[NV]) {
        if constexpr (NV == 1) {
            b[0] = __ldg(p);
        } else if constexpr (NV == 2) {
            const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
            b[0] = t.x; b[1] = t.y;
        } else {
#pragma unroll
            for (int i = 0; i < NV / 4; ++i) {
                const float4 t = __ldg(reinterpret_cast<const float4 *>(p) + i);
                b[4 * i] = t.x; b[4 * i + 1] = t.y; b[4 * i + 2] = t.z; b[4 * i + 3] = t.w;
            }
        }
    }
    __device__ static void load_plain(const float *p, float (&b)[NV]) {
        if constexpr (NV == 1) {
            b[0] = *p;
        } else if constexpr (NV == 2) {
            const float2 t = *reinterpret_cast<const float2 *>(p);
            b[0] = t.x; b[1] = t.y;
        } else {
#pragma unroll
            for (int i = 0; i < NV / 4; ++i) {
                const float4 t = reinterpret_cast<const float4 *>(p)[i];
                b[4 * i] = t.x; b[4 * i + 1] = t.y; b[4 * i + 2] = t.z; b[4 * i + 3] = t.w;
            }
        }
    }
    __device__ static void store(float *p, const float (&o)[NV]) {
        if constexpr (NV == 1) {
            *p = o[0];
        } else if constexpr (NV == 2) {
            *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
        } else {
#pragma unroll
            for (int i = 0; i < NV / 4; ++i)
                reinterpret_cast<float4 *>(p)[i] = make_float4(o[4 * i], o[4 * i + 1], o[4 * i + 2], o[4 * i + 3]);
        }
    }
};

// 16-bit element types: NV elements are NV*2 bytes, loaded as one 2/4/8/16-byte word.
template <class H> struct Half2Of;
template <> struct Half2Of<__nv_bfloat16> {
    using T2 = __nv_bfloat162;
    __device__ static float2 f2(T2 v) { return __bfloat1622float2(v); }
    __device__ static T2 from(float a, float b) { return __floats2bfloat162_rn(a, b); }
};
template <> struct Half2Of<__half> {
    using T2 = __half2;
    __device__ static float2 f2(T2 v) { return __half22float2(v); }
    __device__ static T2 from(float a, float b) { return __floats2half2_rn(a, b); }
};

template <int NV, class H> struct VecIO16 {
    using H2 = Half2Of<H>;
    using T2 = typename H2::T2;
    template <bool NC>
    __device__ static void load_t(const H *p, float (&b)[NV]) {
        if constexpr (NV == 1) {
            b[0] = DT<H>::to_f32(NC ? __ldg(p) : *p);
        } else if constexpr (NV == 2) {
            const uint32_t w = NC ? __ldg(reinterpret_cast<const unsigned int *>(p)) : *reinterpret_cast<const uint32_t *>(p);
            const float2 f = H2::f2(*reinterpret_cast<const T2 *>(&w));
            b[0] = f.x; b[1] = f.y;
        } else if constexpr (NV == 4) {
            const uint2 w = NC ? __ldg(reinterpret_cast<const uint2 *>(p)) : *reinterpret_cast<const uint2 *>(p);
            const float2 f0 = H2::f2(*reinterpret_cast<const T2 *>(&w.x));
            const float2 f1 = H2::f2(*reinterpret_cast<const T2 *>(&w.y));
            b[0] = f0.x; b[1] = f0.y; b[2] = f1.x; b[3] = f1.y;
        } else {
            const uint4 w = NC ? __ldg(reinterpret_cast<const uint4 *>(p)) : *reinterpret_cast<const uint4 *>(p);
            const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float2 f = H2::f2(*reinterpret_cast<const T2 *>(&ws[i]));
                b[2 * i] = f.x; b[2 * i + 1] = f.y;
            }
        }
    }
    __device__ static void load(const H *__restrict__ p, float (&b)[NV]) { load_t<true>(p, b); }
    __device__ static void load_plain(const H *p, float (&b)[NV]) { load_t<false>(p, b); }
    __device__ static void store(H *p, const float (&o)[NV]) {
        if constexpr (NV == 1) {
            *p = DT<H>::from_f32(o[0]);
        } else {
            T2 t[NV / 2];
#pragma unroll
            for (int i = 0; i < NV / 2; ++i) t[i] = H2::from(o[2 * i], o[2 * i + 1]);
            if constexpr (NV == 2) *reinterpret_cast<T2 *>(p) = t[0];
            else if constexpr (NV == 4) *reinterpret_cast<uint2 *>(p) = *reinterpret_cast<const uint2 *>(t);
            else *reinterpret_cast<uint4 *>(p) = *reinterpret_cast<const uint4 *>(t);
        }
    }
};
template <int NV> struct VecIO<NV, __nv_bfloat16> : VecIO16<NV, __nv_bfloat16> {};
template <int NV> struct VecIO<NV, __half> : VecIO16<NV, __half> {};

// C of a 512-column strip with 16-bit B (NV = 16): lane l holds columns 8l .. 8l + 7 of each
// 256-column half (element j is column 256 (j / 8) + 8l + j % 8), as its B row segments.
template <int NV, class TC> struct HalvesIO {
    static_assert(NV == 16, "two 256-column halves of 8 columns a lane");
    __device__ static void load(const TC *__restrict__ p, float (&b)[NV]) {
        float h[2][8];
        VecIO<8, TC>::load(p, h[0]);
        VecIO<8, TC>::load(p + 256, h[1]);
#pragma unroll
        for (int j = 0; j < NV; ++j) b[j] = h[j >> 3][j & 7];
    }
    __device__ static void load_plain(const TC *p, float (&b)[NV]) {
        float h[2][8];
        VecIO<8, TC>::load_plain(p, h[0]);
        VecIO<8, TC>::load_plain(p + 256, h[1]);
#pragma unroll
        for (int j = 0; j < NV; ++j) b[j] = h[j >> 3][j & 7];
    }
    __device__ static void store(TC *p, const float (&o)[NV]) {
        float h[2][8];
#pragma unroll
        for (int j = 0; j < NV; ++j) h[j >> 3][j & 7] = o[j];
        VecIO<8, TC>::store(p, h[0]);
        VecIO<8, TC>::store(p + 256, h[1]);
    }
};

// ------------------------------------------------------------------ B row sources
// One lane's NV columns of a B row in registers: FP32 as floats; 16-bit B as the packed raw values
// (pairs per 32-bit word), which the mixed-precision FMA (fma_vb) widens itself.
template <int NV, class TB> struct BSeg { float f[NV]; };
template <int NV> struct BSeg<NV, __nv_bfloat16> { uint32_t w[(NV + 1) / 2]; };
template <int NV> struct BSeg<NV, __half> { uint32_t w[(NV + 1) / 2]; };

// GlobalB reads the B rows of one lane's columns through L1/L2.
template <int NV, class TB> struct GlobalB {
    const TB *p;  // B + this lane's first column
    int64_t ld;
    bool valid;   // NV == 1 lanes past the last column read zeros and never store
    __device__ __forceinline__ void load(int k, float (&b)[NV]) const {
        if constexpr (NV == 1) {
            b[0] = valid ? DT<TB>::to_f32(__ldg(p + (int64_t)k * ld)) : 0.0f;
        } else {
            VecIO<NV, TB>::load(p + (int64_t)k * ld, b);
        }
    }
    // 16-bit B, NV = 8 and 16 (256- and 512-column strips): the lane's 8 columns of each
    // 256-column part as 4 packed words (for the mixed-precision FMA of run_group_wide)
    __device__ __forceinline__ void load_raw(int k, uint32_t (&w)[NV / 2]) const {
        static_assert(sizeof(TB) == 2 && (NV == 8 || NV == 16), "packed B rows are 16-bit, 8 columns a lane and part");
#pragma unroll
        for (int i = 0; i < NV / 8; ++i) {
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p + (int64_t)k * ld + 256 * i));
            w[4 * i] = v.x; w[4 * i + 1] = v.y; w[4 * i + 2] = v.z; w[4 * i + 3] = v.w;
        }
    }
    __device__ __forceinline__ void load(int k, BSeg<NV, TB> &b) const {
        if constexpr (sizeof(TB) == 4) {
            load(k, b.f);
        } else {
            const TB *q = p + (int64_t)k * ld;
            if constexpr (NV == 1) {
                b.w[0] = valid ? (uint32_t)__ldg(reinterpret_cast<const unsigned short *>(q)) : 0u;
            } else if constexpr (NV == 2) {
                b.w[0] = __ldg(reinterpret_cast<const unsigned int *>(q));
            } else if constexpr (NV == 4) {
                const uint2 v = __ldg(reinterpret_cast<const uint2 *>(q));
                b.w[0] = v.x; b.w[1] = v.y;
            } else {
                const uint4 v = __ldg(reinterpret_cast<const uint4 *>(q));
                b.w[0] = v.x; b.w[1] = v.y; b.w[2] = v.z; b.w[3] = v.w;
            }
        }
    }
};

// FP32 strips of 256 and 512 columns (NV = 8, 16) in the gather kernel.  Lane l holds columns
// 4l .. 4l + 3 of each 128-column quarter of the strip (element j is column 128 (j / 4) + 4l + j % 4),
// so every 16-byte load or store of the warp covers 512 contiguous bytes: whole 128-byte lines, one
// L1 wavefront each, where NV contiguous columns a lane would spread each instruction over 32 NV
// bytes.  At high sparsity an entry's index, value and address work is then shared by 8 or 16
// columns a lane instead of 4.
template <int NV> struct WideIO {
    static_assert(NV % 4 == 0, "wide strips hold whole float4 quarters");
    __device__ static void load(const float *__restrict__ p, float (&b)[NV]) {
#pragma unroll
        for (int i = 0; i < NV / 4; ++i) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(p + 128 * i));
            b[4 * i] = t.x; b[4 * i + 1] = t.y; b[4 * i + 2] = t.z; b[4 * i + 3] = t.w;
        }
    }
    __device__ static void load_plain(const float *p, float (&b)[NV]) {
#pragma unroll
        for (int i = 0; i < NV / 4; ++i) {
            const float4 t = *reinterpret_cast<const float4 *>(p + 128 * i);
            b[4 * i] = t.x; b[4 * i + 1] = t.y; b[4 * i + 2] = t.z; b[4 * i + 3] = t.w;
        }
    }
    __device__ static void store(float *p, const float (&o)[NV]) {
#pragma unroll
        for (int i = 0; i < NV / 4; ++i)
            *reinterpret_cast<float4 *>(p + 128 * i) = make_float4(o[4 * i], o[4 * i + 1], o[4 * i + 2], o[4 * i + 3]);
    }
};

template <int NV> struct GlobalBWide {
    const float *p;  // B + this lane's first column
    int64_t ld;
    bool valid;      // wide strips are whole: every lane is valid
    __device__ __forceinline__ void load(int k, float (&b)[NV]) const { WideIO<NV>::load(p + (int64_t)k * ld, b); }
    __device__ __forceinline__ void load(int k, BSeg<NV, float> &b) const { load(k, b.f); }
};

// ------------------------------------------------------------------ metadata streams
// A unit's column indices, values and nkern_counts are each read front to back.  A Stream keeps a
// 64-element window of one of them in two registers per lane (element i of the window is lane
// i % 32 of cur / nxt) and refills 32 elements as soon as 32 have been consumed, so every refill
// load has 32 elements of work to hide behind.  All lanes hold the same position (warp-uniform).
template <class T> struct RawOf { using R = T; };
template <> struct RawOf<__nv_bfloat16> { using R = unsigned short; };
template <> struct RawOf<__half> { using R = unsigned short; };

template <class T> struct Stream {
    using R = typename RawOf<T>::R;
    const R *p;      // next element to load into the window
    int64_t left;    // elements from p on that belong to the array
    R cur, nxt;      // window elements [0, 32) and [32, 64)
    int pos;         // window position of the next element to take

    __device__ __forceinline__ static R load1(const R *q, int64_t left, int lane) {
        return lane < left ? __ldg(q + lane) : R(0);
    }
    __device__ __forceinline__ void init(const T *base, int64_t n) {
        const int lane = threadIdx.x & 31;
        p = reinterpret_cast<const R *>(base);
        left = n;
        cur = load1(p, left, lane);
        nxt = load1(p + 32, left - 32, lane);
        p += 64;
        left -= 64;
        pos = 0;
    }
    // Make sure the next `need` (<= 32) elements are inside the window.
    __device__ __forceinline__ void ensure() {
        if (pos >= 32) {
            cur = nxt;
            nxt = load1(p, left, threadIdx.x & 31);
            p += 32;
            left -= 32;
            pos -= 32;
        }
    }
    __device__ __forceinline__ R at(int i) const {  // window element pos + i (pos + i < 64)
        const int w = pos + i;
        return __shfl_sync(0xffffffffu, w < 32 ? cur : nxt, w & 31);
    }
};

__device__ __forceinline__ float raw_to_f32(float v) { return v; }
template <class TV> __device__ __forceinline__ float val_f32(typename RawOf<TV>::R r) {
    if constexpr (std::is_same<TV, float>::value) return r;
    else return DT<TV>::to_f32(*reinterpret_cast<const TV *>(&r));
}

// ------------------------------------------------------------------ nanokernel loops
// acc[r] += value * b for every set row r of PAT (values in ascending row order, starting at
// window offset vbase of the value stream).
template <int PAT, int MR, int NV, class TV>
__device__ __forceinline__ void fma_entry(const Stream<TV> &vs, const int vbase, const float (&b)[NV],
                                          float (&acc)[MR][NV]) {
    int q = 0;
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        if ((PAT >> r) & 1) {
            const float a = val_f32<TV>(vs.at(vbase + q));
            ++q;
#pragma unroll
            for (int j = 0; j < NV; ++j) acc[r][j] = fmaf(a, b[j], acc[r][j]);
        }
    }
}

// n entries of one nanokernel id, U at a time: U B-row loads are issued before their FMAs.
template <int PAT, int MR, int NV, class TV, class BL>
__device__ __forceinline__ void run_group(int n, Stream<int32_t> &cs, Stream<TV> &vs, const BL &bl,
                                          float (&acc)[MR][NV]) {
    constexpr int PC = cpopc(PAT);
    constexpr int U0 = NV >= 4 ? 2 : 4;
    constexpr int U = (U0 * PC <= 32) ? U0 : (32 / PC);
    for (; n >= U; n -= U) {
        cs.ensure();
        vs.ensure();
        float b[U][NV];
#pragma unroll
        for (int u = 0; u < U; ++u) bl.load(cs.at(u), b[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) fma_entry<PAT, MR, NV, TV>(vs, u * PC, b[u], acc);
        cs.pos += U;
        vs.pos += U * PC;
    }
    for (; n > 0; --n) {
        cs.ensure();
        vs.ensure();
        float b[NV];
        bl.load(cs.at(0), b);
        fma_entry<PAT, MR, NV, TV>(vs, 0, b, acc);
        cs.pos += 1;
        vs.pos += PC;
    }
}

// M_r = 6 and 8 have 63 and 255 patterns; compiling a loop per pattern takes minutes, so M_r = 8
// specialises the single rows and the nanokernels of the reference's M_r = 8 "orig" (400fa) and
// "alt" (747f9) sets (tools/paper/configs.py:84-87), M_r = 6 the single rows, and any other
// pattern runs through the nibble path (rows 0-3, then rows 4-7, one 16-way switch each).
template <int MR>
__host__ __device__ constexpr bool fast_pattern(int P) {
    if (P <= 0 || P >= (1 << MR)) return false;
    if (MR <= 4) return true;
    if (MR == 6) return (P & (P - 1)) == 0;  // single rows; other M_r = 6 patterns take the nibble path
    switch (P) {
    case 1: case 2: case 4: case 8: case 16: case 32: case 64: case 128:
    case 15: case 60: case 85: case 170: case 195: case 240:
    case 63: case 207: case 243: case 252: case 255:
        return true;
    default:
        return false;
    }
}

// Rows BASE .. BASE+3 of a 4-bit sub-pattern Q (values from window offset vbase).
template <int Q, int BASE, int MR, int NV, class TV>
__device__ __forceinline__ void fma_nibble(const Stream<TV> &vs, const int vbase, const float (&b)[NV],
                                           float (&acc)[MR][NV]) {
    int q = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if (((Q >> r) & 1) && BASE + r < MR) {
            const float a = val_f32<TV>(vs.at(vbase + q));
            ++q;
#pragma unroll
            for (int j = 0; j < NV; ++j) acc[BASE + r][j] = fmaf(a, b[j], acc[BASE + r][j]);
        }
    }
}

// Any M_r = 8 pattern: rows 0-3 then rows 4-7, each through a 16-way switch per entry.
template <int MR, int NV, class TV, class BL>
__device__ __forceinline__ void run_group_nibbles(const int pat, int n, Stream<int32_t> &cs, Stream<TV> &vs,
                                                  const BL &bl, float (&acc)[MR][NV]) {
    if constexpr (MR > 4) {
        const int lo = pat & 15, hi = (pat >> 4) & 15;
        const int plo = __popc(lo), pc = __popc(pat);
        for (; n > 0; --n) {
            cs.ensure();
            vs.ensure();
            float b[NV];
            bl.load(cs.at(0), b);
#define SPREG_NIB_LO(Q) case Q: fma_nibble<Q, 0, MR, NV, TV>(vs, 0, b, acc); break;
#define SPREG_NIB_HI(Q) case Q: fma_nibble<Q, 4, MR, NV, TV>(vs, plo, b, acc); break;
            switch (lo) {
                SPREG_NIB_LO(1) SPREG_NIB_LO(2) SPREG_NIB_LO(3) SPREG_NIB_LO(4) SPREG_NIB_LO(5)
                SPREG_NIB_LO(6) SPREG_NIB_LO(7) SPREG_NIB_LO(8) SPREG_NIB_LO(9) SPREG_NIB_LO(10)
                SPREG_NIB_LO(11) SPREG_NIB_LO(12) SPREG_NIB_LO(13) SPREG_NIB_LO(14) SPREG_NIB_LO(15)
                default: break;
            }
            switch (hi) {
                SPREG_NIB_HI(1) SPREG_NIB_HI(2) SPREG_NIB_HI(3) SPREG_NIB_HI(4) SPREG_NIB_HI(5)
                SPREG_NIB_HI(6) SPREG_NIB_HI(7) SPREG_NIB_HI(8) SPREG_NIB_HI(9) SPREG_NIB_HI(10)
                SPREG_NIB_HI(11) SPREG_NIB_HI(12) SPREG_NIB_HI(13) SPREG_NIB_HI(14) SPREG_NIB_HI(15)
                default: break;
            }
#undef SPREG_NIB_LO
#undef SPREG_NIB_HI
            cs.pos += 1;
            vs.pos += pc;
        }
    }
}

#define SPREG_C4(F, b) F((b)) F((b) + 1) F((b) + 2) F((b) + 3)
#define SPREG_C16(F, b) SPREG_C4(F, b) SPREG_C4(F, (b) + 4) SPREG_C4(F, (b) + 8) SPREG_C4(F, (b) + 12)
#define SPREG_C64(F, b) SPREG_C16(F, b) SPREG_C16(F, (b) + 16) SPREG_C16(F, (b) + 32) SPREG_C16(F, (b) + 48)

template <int MR, int NV, class TV, class BL>
__device__ __forceinline__ void dispatch_group(const int pat, const int n, Stream<int32_t> &cs, Stream<TV> &vs,
                                               const BL &bl, float (&acc)[MR][NV]) {
#define SPREG_CASE(P)                                                                  \
    case (P):                                                                          \
        if constexpr (fast_pattern<MR>(P)) {                                           \
            run_group<fast_pattern<MR>(P) ? (P) : 1, MR, NV, TV, BL>(n, cs, vs, bl, acc); \
            return;                                                                    \
        }                                                                              \
        break;
    switch (pat) {
        SPREG_C64(SPREG_CASE, 0)
        SPREG_C64(SPREG_CASE, 64)
        SPREG_C64(SPREG_CASE, 128)
        SPREG_C64(SPREG_CASE, 192)
    default:
        break;
    }
#undef SPREG_CASE
    if constexpr (MR > 4) run_group_nibbles<MR, NV, TV, BL>(pat, n, cs, vs, bl, acc);
}

// ------------------------------------------------------------------ one row panel x one strip
template <int MR, int NV, class TV, class TC, class BL>
__device__ __forceinline__ void process_panel(const ExecParams &p, const int64_t gp, const int64_t col0,
                                              const bool valid, const BL &bl) {
    constexpr bool SCALED = std::is_same<TV, __half>::value;
    const int64_t row0 = gp * MR;
    TC *C = reinterpret_cast<TC *>(p.C);
    float acc[MR][NV];
#pragma unroll
    for (int r = 0; r < MR; ++r)
#pragma unroll
        for (int j = 0; j < NV; ++j) acc[r][j] = 0.0f;
    if (!SCALED && p.load_c && valid) {
#pragma unroll
        for (int r = 0; r < MR; ++r)
            if (row0 + r < p.M) VecIO<NV, TC>::load_plain(C + (row0 + r) * p.ldc + col0, acc[r]);
    }
    for (int64_t tj = 0; tj < p.T; ++tj) {
        const spreg_panel_desc d = p.descs[unit_index(gp, tj, p.ppt, p.T, p.P)];
        if (d.num_cols == 0) continue;
        Stream<int32_t> ks, cs;
        Stream<TV> vs;
        ks.init(reinterpret_cast<const int32_t *>(p.arena + d.counts_off), p.nk);
        cs.init(reinterpret_cast<const int32_t *>(p.arena + d.cols_off), d.num_cols);
        vs.init(reinterpret_cast<const TV *>(p.arena + d.values_off), d.num_values);
        for (int id = 0; id < p.nk; ++id) {
            ks.ensure();
            const int n = ks.at(0);
            ks.pos += 1;
            if (n == 0) continue;
            dispatch_group<MR, NV, TV, BL>(p.id_pattern[id], n, cs, vs, bl, acc);
        }
    }
    if (!valid) return;
    const float s = SCALED ? p.scales[gp] : 1.0f;
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        if (row0 + r >= p.M) continue;
        TC *cp = C + (row0 + r) * p.ldc + col0;
        float o[NV];
#pragma unroll
        for (int j = 0; j < NV; ++j) o[j] = acc[r][j];
        if (SCALED) {
            if (p.load_c) {
                float cin[NV];
                VecIO<NV, TC>::load_plain(cp, cin);
#pragma unroll
                for (int j = 0; j < NV; ++j) o[j] = fmaf(o[j], s, cin[j]);
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) o[j] = o[j] * s;
            }
        }
        if (p.epilogue == SPREG_EPILOGUE_RELU) {
#pragma unroll
            for (int j = 0; j < NV; ++j) o[j] = fmaxf(o[j], 0.0f);
        }
        VecIO<NV, TC>::store(cp, o);
    }
}

// ------------------------------------------------------------------ kernels
// B through L1/L2: one warp per (row panel, strip); grid (panel groups, strips).
template <int MR, int NV, class TV, class TB, class TC>
__global__ void __launch_bounds__(256, 1) exec_kernel(const __grid_constant__ ExecParams p) {
    const int lane = threadIdx.x & 31;
    const int64_t gp = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gp >= p.P) return;
    const int64_t col0 = p.col_begin + (int64_t)blockIdx.y * (32 * NV) + (int64_t)lane * NV;
    const bool valid = col0 < p.N;  // NV > 1 launches cover whole strips only
    GlobalB<NV, TB> bl{reinterpret_cast<const TB *>(p.B) + col0, p.ldb, valid};
    process_panel<MR, NV, TV, TC>(p, gp, col0, valid, bl);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase; false after `limit` polls (then *status records `code`).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase, int *status, int code,
                                                  uint32_t limit = 1u << 22) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    if (status) atomicCAS(status, 0, code);
    return false;
}

// ================================================================== execution-layout executor
__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ uint4 lds_u128(uint32_t a) {
    uint4 v;
    asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a));
    return v;
}
__device__ __forceinline__ unsigned short lds_u16(uint32_t a) {
    unsigned short v;
    asm volatile("ld.shared.b16 %0, [%1];" : "=h"(v) : "r"(a));
    return v;
}
template <class TV> __device__ __forceinline__ float word_val(uint32_t w, int half) {
    if constexpr (sizeof(TV) == 4) {
        return __uint_as_float(w);
    } else if constexpr (std::is_same<TV, __nv_bfloat16>::value) {
        // BF16 is the upper half of an FP32 word: the widening is exact, one logical op per value
        return __uint_as_float(half ? (w & 0xFFFF0000u) : (w << 16));
    } else {
        const unsigned short h = (unsigned short)(half ? (w >> 16) : (w & 0xFFFFu));
        return DT<TV>::to_f32(*reinterpret_cast<const TV *>(&h));
    }
}
// Mixed-precision FMA (fma.rn.f32.bf16 / .f16): d = a * b + c with a, b the 16-bit halves HA / HB
// (0 = low) of two 32-bit words and c, d FP32.  The product of two 16-bit values is exact in FP32,
// so the result equals fmaf(float(a), float(b), c) bit for bit, without the two widening ops.
#define SPREG_FMA_MIXED(T, A, B)                                                                     \
    asm("{\n\t.reg .b16 a0, a1, b0, b1;\n\tmov.b32 {a0, a1}, %1;\n\tmov.b32 {b0, b1}, %2;\n\t" \
        "fma.rn.f32." T " %0, " A ", " B ", %3;\n\t}"                                            \
        : "=f"(d) : "r"(aw), "r"(bw), "f"(c))
template <class TV, int HA, int HB>
__device__ __forceinline__ float fma_mixed(const uint32_t aw, const uint32_t bw, const float c) {
    float d;
    if constexpr (std::is_same<TV, __nv_bfloat16>::value) {
        if constexpr (HA == 0 && HB == 0) SPREG_FMA_MIXED("bf16", "a0", "b0");
        else if constexpr (HA == 0) SPREG_FMA_MIXED("bf16", "a0", "b1");
        else if constexpr (HB == 0) SPREG_FMA_MIXED("bf16", "a1", "b0");
        else SPREG_FMA_MIXED("bf16", "a1", "b1");
    } else {
        if constexpr (HA == 0 && HB == 0) SPREG_FMA_MIXED("f16", "a0", "b0");
        else if constexpr (HA == 0) SPREG_FMA_MIXED("f16", "a0", "b1");
        else if constexpr (HB == 0) SPREG_FMA_MIXED("f16", "a1", "b0");
        else SPREG_FMA_MIXED("f16", "a1", "b1");
    }
    return d;
}
#undef SPREG_FMA_MIXED

// acc + a * b[j]: a = half `ha` of value word aw (the word itself for FP32), b[j] = column j of the
// lane's B segment.  ha and j are compile-time after unrolling.
template <class TV, int NV>
__device__ __forceinline__ float fma_vb(const uint32_t aw, const int ha, const BSeg<NV, TV> &b, const int j,
                                        const float c) {
    if constexpr (sizeof(TV) == 4) {
        return fmaf(__uint_as_float(aw), b.f[j], c);
    } else {
        const uint32_t bw = b.w[j >> 1];
        if (ha == 0) return (j & 1) ? fma_mixed<TV, 0, 1>(aw, bw, c) : fma_mixed<TV, 0, 0>(aw, bw, c);
        return (j & 1) ? fma_mixed<TV, 1, 1>(aw, bw, c) : fma_mixed<TV, 1, 0>(aw, bw, c);
    }
}
// Column j of a B segment as FP32 (paths that multiply by an FP32 value).
template <class TV, int NV> __device__ __forceinline__ float bseg_f32(const BSeg<NV, TV> &b, const int j) {
    if constexpr (sizeof(TV) == 4) return b.f[j];
    else return word_val<TV>(b.w[j >> 1], j & 1);
}

template <class TV> __device__ __forceinline__ float lds_val(uint32_t a) {
    if constexpr (sizeof(TV) == 4) return __uint_as_float(lds_u32(a));
    else return word_val<TV>(lds_u16(a), 0);
}

__device__ __forceinline__ uint2 lds_u64(uint32_t a) {
    uint2 v;
    asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
    return v;
}

// The FMAs of one step (4 entries) of a group of pattern PAT: the step's 4 * PC values are PC
// broadcast loads of 16 (FP32) or 8 (16-bit) bytes; entry u's values follow in ascending row
// order.  FULL steps have 4 entries; the last step of a group has m < 4 (entries u >= m skipped).
template <int PAT, int MR, int NV, class TV, bool FULL>
__device__ __forceinline__ void step_fma(const uint32_t vs, const int m, const BSeg<NV, TV> (&b)[4],
                                         float (&acc)[MR][NV]) {
    constexpr int PC = cpopc(PAT);
    constexpr int VB = (int)sizeof(TV);
    uint32_t vw[PC * VB];
#pragma unroll
    for (int i = 0; i < PC; ++i) {
        if constexpr (VB == 4) {
            const uint4 t = lds_u128(vs + 16u * i);
            vw[4 * i] = t.x; vw[4 * i + 1] = t.y; vw[4 * i + 2] = t.z; vw[4 * i + 3] = t.w;
        } else {
            const uint2 t = lds_u64(vs + 8u * i);
            vw[2 * i] = t.x; vw[2 * i + 1] = t.y;
        }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        if (FULL || u < m) {
            int q = 0;
#pragma unroll
            for (int r = 0; r < MR; ++r) {
                if ((PAT >> r) & 1) {
                    const int vi = u * PC + q;
                    ++q;
#pragma unroll
                    for (int j = 0; j < NV; ++j)
                        acc[r][j] = fma_vb<TV, NV>(vw[vi * VB / 4], (vi * VB / 2) & 1, b[u], j, acc[r][j]);
                }
            }
        }
    }
}

// Rows BASE .. BASE+3 of the 4-bit sub-pattern Q of one entry (values from shared address va).
template <int Q, int BASE, int MR, int NV, class TV>
__device__ __forceinline__ void fma_nibble_x(uint32_t va, const BSeg<NV, TV> &b, float (&acc)[MR][NV]) {
    int q = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if (((Q >> r) & 1) && BASE + r < MR) {
            const float a = lds_val<TV>(va + (uint32_t)(q * sizeof(TV)));
            ++q;
#pragma unroll
            for (int j = 0; j < NV; ++j) acc[BASE + r][j] = fmaf(a, bseg_f32<TV, NV>(b, j), acc[BASE + r][j]);
        }
    }
}

// One step of a pattern without its own FMA block (M_r 6 and 8): entry by entry, rows 0-3 then
// rows 4-7 through 16-way switches.
template <int MR, int NV, class TV>
__device__ __forceinline__ void step_fma_nibbles(const int pat, const uint32_t vs, const int m, const BSeg<NV, TV> (&b)[4],
                                                 float (&acc)[MR][NV]) {
    if constexpr (MR > 4) {
        const int lo = pat & 15, hi = (pat >> 4) & 15;
        const uint32_t plo = (uint32_t)(__popc(lo) * sizeof(TV)), ent = (uint32_t)(__popc(pat) * sizeof(TV));
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (u < m) {
                const uint32_t va = vs + ent * u;
#define SPREG_XLO(Q) case Q: fma_nibble_x<Q, 0, MR, NV, TV>(va, b[u], acc); break;
#define SPREG_XHI(Q) case Q: fma_nibble_x<Q, 4, MR, NV, TV>(va + plo, b[u], acc); break;
                switch (lo) {
                    SPREG_XLO(1) SPREG_XLO(2) SPREG_XLO(3) SPREG_XLO(4) SPREG_XLO(5) SPREG_XLO(6) SPREG_XLO(7)
                    SPREG_XLO(8) SPREG_XLO(9) SPREG_XLO(10) SPREG_XLO(11) SPREG_XLO(12) SPREG_XLO(13) SPREG_XLO(14)
                    SPREG_XLO(15)
                    default: break;
                }
                switch (hi) {
                    SPREG_XHI(1) SPREG_XHI(2) SPREG_XHI(3) SPREG_XHI(4) SPREG_XHI(5) SPREG_XHI(6) SPREG_XHI(7)
                    SPREG_XHI(8) SPREG_XHI(9) SPREG_XHI(10) SPREG_XHI(11) SPREG_XHI(12) SPREG_XHI(13) SPREG_XHI(14)
                    SPREG_XHI(15)
                    default: break;
                }
#undef SPREG_XLO
#undef SPREG_XHI
            }
        }
    }
}

// The FMA block of one step, selected by one uniform switch on the pattern.
template <int MR, int NV, class TV, bool FULL>
__device__ __forceinline__ void step_dispatch(const int pat, const uint32_t vs, const int m, const BSeg<NV, TV> (&b)[4],
                                              float (&acc)[MR][NV]) {
    bool done = false;
#define SPREG_CASE(P)                                                                \
    case (P):                                                                        \
        if constexpr (fast_pattern<MR>(P)) {                                         \
            step_fma<fast_pattern<MR>(P) ? (P) : 1, MR, NV, TV, FULL>(vs, m, b, acc); \
            done = true;                                                             \
        }                                                                            \
        break;
    switch (pat) {
        SPREG_C64(SPREG_CASE, 0)
        SPREG_C64(SPREG_CASE, 64)
        SPREG_C64(SPREG_CASE, 128)
        SPREG_C64(SPREG_CASE, 192)
    default:
        break;
    }
#undef SPREG_CASE
    if (!done) step_fma_nibbles<MR, NV, TV>(pat, vs, FULL ? 4 : m, b, acc);
}

// ------------------------------------------------------------------ 256-column strips (NV = 8)
// With NV = 8 a step of 4 entries runs as two halves of 2 entries, so that only 2 B rows of 8
// columns are live beside the 4 x 8 accumulators.  M_r <= 4 (every pattern has its own FMA block).
// Values and B stay packed as 16-bit pairs in 32-bit words: the mixed-precision FMA
// (fma.rn.f32.bf16 / .f16: 16-bit a and b, FP32 c and d) widens its operands itself.  The product
// of two 16-bit values is exact in FP32, so each step equals fmaf(float(a), float(b), c).

// 2 entries of pattern PAT: B rows as packed words b[u][NV / 2], values from shared address vs
// (2 x PC 16-bit values, PC words; a half starts 4 * PC bytes into its step).
template <int PAT, int MR, int NV, class TV, bool FULL, int I0 = 0>
__device__ __forceinline__ void half_fma(const uint32_t vs, const int m, const uint32_t (&b)[2][NV / 2],
                                         float (&acc)[MR][NV]) {
    constexpr int PC = cpopc(PAT);
    static_assert(sizeof(TV) == 2 && MR <= 4, "256-column strips take 16-bit values and M_r <= 4");
    uint32_t vw[PC];
#pragma unroll
    for (int i = 0; i < PC; ++i) vw[i] = lds_u32(vs + 4u * i);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        if (FULL || u < m) {
            int q = 0;
#pragma unroll
            for (int r = 0; r < MR; ++r) {
                if ((PAT >> r) & 1) {
                    const int vi = u * PC + q;
                    ++q;
#pragma unroll
                    for (int j = 0; j < NV; j += 2) {
                        if (vi & 1) {
                            acc[r][j] = fma_mixed<TV, 1, 0>(vw[vi >> 1], b[u][j >> 1], acc[r][j]);
                            acc[r][j + 1] = fma_mixed<TV, 1, 1>(vw[vi >> 1], b[u][j >> 1], acc[r][j + 1]);
                        } else {
                            acc[r][j] = fma_mixed<TV, 0, 0>(vw[vi >> 1], b[u][j >> 1], acc[r][j]);
                            acc[r][j + 1] = fma_mixed<TV, 0, 1>(vw[vi >> 1], b[u][j >> 1], acc[r][j + 1]);
                        }
                    }
                }
            }
        }
    }
}

// The same with the pattern known at run time (groups of patterns without their own loop).
template <int MR, int NV, class TV, bool FULL>
__device__ __forceinline__ void half_dispatch(const int pat, const uint32_t vs, const int m, const uint32_t (&b)[2][NV / 2],
                                              float (&acc)[MR][NV]) {
#define SPREG_HCASE(P)                                                                          \
    case (P):                                                                                   \
        if constexpr ((P) > 0 && (P) < (1 << MR)) half_fma<(P), MR, NV, TV, FULL>(vs, m, b, acc); \
        break;
    switch (pat) {
        SPREG_C16(SPREG_HCASE, 0)
    default:
        break;
    }
#undef SPREG_HCASE
}

// n entries of one group at NV = 8; PAT > 0 is the group's pattern known at compile time, PAT = 0
// dispatches on `pat` once per half step.  The B rows are loaded before the FMA block is chosen
// (a switch around whole steps spilled).
template <int PAT, int MR, int NV, class TV, class BL>
__device__ __forceinline__ void run_group_wide(const int pat, const int n, uint32_t cs, uint32_t vs, const BL &bl,
                                               float (&acc)[MR][NV]) {
    const uint32_t pc = PAT > 0 ? (uint32_t)cpopc(PAT) : (uint32_t)__popc(pat);
    const uint32_t vhalf = 2u * (uint32_t)sizeof(TV) * pc, vstep = 2u * vhalf;
    auto half = [&](uint32_t v, int m, const uint32_t (&b)[2][NV / 2], auto full_tag) {
        constexpr bool FULL = decltype(full_tag)::value;
        if constexpr (PAT > 0) half_fma<PAT, MR, NV, TV, FULL>(v, m, b, acc);
        else half_dispatch<MR, NV, TV, FULL>(pat, v, m, b, acc);
    };
    const int full = n >> 2;
    uint4 k4 = full > 0 ? lds_u128(cs) : make_uint4(0, 0, 0, 0);
#pragma unroll 1
    for (int s = 0; s < full; ++s) {
        const uint4 kk = k4;
        cs += 16u;
        if (s + 1 < full) k4 = lds_u128(cs);
        uint32_t b[2][NV / 2];
        bl.load_raw((int)kk.x, b[0]);
        bl.load_raw((int)kk.y, b[1]);
        half(vs, 2, b, std::true_type{});
        bl.load_raw((int)kk.z, b[0]);
        bl.load_raw((int)kk.w, b[1]);
        half(vs + vhalf, 2, b, std::true_type{});
        vs += vstep;
    }
    const int m = n & 3;
    if (m) {
        const uint4 kk = lds_u128(cs);
        uint32_t b[2][NV / 2];
        bl.load_raw((int)kk.x, b[0]);
        if (m > 1) bl.load_raw((int)kk.y, b[1]);
        half(vs, m < 2 ? m : 2, b, std::false_type{});
        if (m > 2) {
            bl.load_raw((int)kk.z, b[0]);
            half(vs + vhalf, m - 2, b, std::false_type{});
        }
    }
}

// n entries of one group: full steps of 4 entries (one 16-byte broadcast load of column indices,
// 4 B rows, the pattern's FMA block), then one predicated step for the last n % 4 entries.
// A group of a pattern known at compile time: no per-step dispatch.
template <int PAT, int MR, int NV, class TV, class BL>
__device__ __forceinline__ void run_group_pat(const int n, uint32_t cs, uint32_t vs, const BL &bl,
                                              float (&acc)[MR][NV]) {
    constexpr uint32_t VSTEP = 4u * (uint32_t)sizeof(TV) * (uint32_t)cpopc(PAT);
    const int full = n >> 2;
    if constexpr (NV >= 8 && sizeof(TV) == 2) {
        run_group_wide<PAT, MR, NV, TV>(PAT, n, cs, vs, bl, acc);
        return;
    } else if constexpr (NV >= 4) {
        // registers are short for a second B set: prefetch only the next step's column indices
        uint4 k4 = full > 0 ? lds_u128(cs) : make_uint4(0, 0, 0, 0);
#pragma unroll 1
        for (int s = 0; s < full; ++s) {
            BSeg<NV, TV> b[4];
            bl.load((int)k4.x, b[0]);
            bl.load((int)k4.y, b[1]);
            bl.load((int)k4.z, b[2]);
            bl.load((int)k4.w, b[3]);
            cs += 16u;
            if (s + 1 < full) k4 = lds_u128(cs);
            step_fma<PAT, MR, NV, TV, true>(vs, 4, b, acc);
            vs += VSTEP;
        }
    } else if (full > 0) {
        // software pipeline: the next step's column indices and B rows load before this step's FMAs
        uint4 k4 = lds_u128(cs);
        BSeg<NV, TV> b[4];
        bl.load((int)k4.x, b[0]);
        bl.load((int)k4.y, b[1]);
        bl.load((int)k4.z, b[2]);
        bl.load((int)k4.w, b[3]);
#pragma unroll 1
        for (int s = 0; s < full; ++s) {
            cs += 16u;
            BSeg<NV, TV> bn[4];
            if (s + 1 < full) {
                k4 = lds_u128(cs);
                bl.load((int)k4.x, bn[0]);
                bl.load((int)k4.y, bn[1]);
                bl.load((int)k4.z, bn[2]);
                bl.load((int)k4.w, bn[3]);
            }
            step_fma<PAT, MR, NV, TV, true>(vs, 4, b, acc);
            vs += VSTEP;
#pragma unroll
            for (int u = 0; u < 4; ++u) b[u] = bn[u];
        }
    }
    const int m = n & 3;
    if (m) {
        const uint4 k4 = lds_u128(cs);
        const int ks[4] = {(int)k4.x, (int)k4.y, (int)k4.z, (int)k4.w};
        BSeg<NV, TV> b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (u < m) bl.load(ks[u], b[u]);
        step_fma<PAT, MR, NV, TV, false>(vs, m, b, acc);
    }
}

// With HOT (the shared-memory B-tile kernel, which has the registers for it), the single rows and the
// all-rows nanokernel of M_r = 2 and 4 -- the common groups at high sparsity, and the set the
// histogram-based selection picks -- run their own loop; every other pattern dispatches per step.
template <int MR, int NV, class TV, bool HOT = false, class BL>
__device__ __forceinline__ void run_group_x(const int pat, const int n, uint32_t cs, uint32_t vs, const BL &bl,
                                            float (&acc)[MR][NV]) {
    if constexpr (HOT && (MR == 2 || MR == 4)) {
        switch (pat) {
        case 1: run_group_pat<1, MR, NV, TV>(n, cs, vs, bl, acc); return;
        case 2: run_group_pat<2, MR, NV, TV>(n, cs, vs, bl, acc); return;
        case (1 << MR) - 1: run_group_pat<(1 << MR) - 1, MR, NV, TV>(n, cs, vs, bl, acc); return;
        default: break;
        }
        if constexpr (MR == 4) {
            switch (pat) {
            case 4: run_group_pat<4, MR, NV, TV>(n, cs, vs, bl, acc); return;
            case 8: run_group_pat<8, MR, NV, TV>(n, cs, vs, bl, acc); return;
            default: break;
            }
        }
    }
    if constexpr (NV >= 8 && sizeof(TV) == 2) {
        run_group_wide<0, MR, NV, TV>(pat, n, cs, vs, bl, acc);
        return;
    }
    const uint32_t vstep = 4u * (uint32_t)sizeof(TV) * (uint32_t)__popc(pat);
    const int full = n >> 2;
#pragma unroll 1
    for (int s = 0; s < full; ++s) {
        const uint4 k4 = lds_u128(cs);
        BSeg<NV, TV> b[4];
        bl.load((int)k4.x, b[0]);
        bl.load((int)k4.y, b[1]);
        bl.load((int)k4.z, b[2]);
        bl.load((int)k4.w, b[3]);
        step_dispatch<MR, NV, TV, true>(pat, vs, 4, b, acc);
        cs += 16u;
        vs += vstep;
    }
    const int m = n & 3;
    if (m) {
        const uint4 k4 = lds_u128(cs);
        const int ks[4] = {(int)k4.x, (int)k4.y, (int)k4.z, (int)k4.w};
        BSeg<NV, TV> b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (u < m) bl.load(ks[u], b[u]);
        step_dispatch<MR, NV, TV, false>(pat, vs, m, b, acc);
    }
}

// C tile of one row panel: load (load_c) / store with scale and epilogue.
template <int MR, int NV, class TV, class TC>
__device__ __forceinline__ void panel_acc_init(const ExecParams &p, int64_t row0, int64_t col0, float (&acc)[MR][NV]) {
    constexpr bool SCALED = std::is_same<TV, __half>::value;
#pragma unroll
    for (int r = 0; r < MR; ++r)
#pragma unroll
        for (int j = 0; j < NV; ++j) acc[r][j] = 0.0f;
    if (!SCALED && p.load_c) {
        const TC *C = reinterpret_cast<const TC *>(p.C);
#pragma unroll
        for (int r = 0; r < MR; ++r)
            if (row0 + r < p.M) VecIO<NV, TC>::load_plain(C + (row0 + r) * p.ldc + col0, acc[r]);
    }
}
template <int MR, int NV, class TV, class TC>
__device__ __forceinline__ void panel_store(const ExecParams &p, int64_t gp, int64_t row0, int64_t col0,
                                            const float (&acc)[MR][NV]) {
    constexpr bool SCALED = std::is_same<TV, __half>::value;
    TC *C = reinterpret_cast<TC *>(p.C);
    const float s = SCALED ? p.scales[gp] : 1.0f;
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        if (row0 + r >= p.M) continue;
        TC *cp = C + (row0 + r) * p.ldc + col0;
        float o[NV];
#pragma unroll
        for (int j = 0; j < NV; ++j) o[j] = acc[r][j];
        if (SCALED) {
            if (p.load_c) {
                float cin[NV];
                VecIO<NV, TC>::load_plain(cp, cin);
#pragma unroll
                for (int j = 0; j < NV; ++j) o[j] = fmaf(o[j], s, cin[j]);
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) o[j] = o[j] * s;
            }
        }
        if (p.epilogue == SPREG_EPILOGUE_RELU) {
#pragma unroll
            for (int j = 0; j < NV; ++j) o[j] = fmaxf(o[j], 0.0f);
        }
        VecIO<NV, TC>::store(cp, o);
    }
}

// ================================================================== batched persistent executor
// One launch runs many SpMMs (problems) of uneven shape.  The work is a list of items
// (problem, row panel, column strip); warps take items from a global counter (zeroed by the host
// before the launch) until the list is exhausted, so every SM stays busy to the end whatever the
// row skew.  For each item the warp bulk-copies the execution blocks of the panel's K-tile units
// into a shared-memory buffer; two buffers per warp keep the next block in flight while the
// current one computes.  Problems of one launch share M_r, the strip width and the data types;
// the problem table travels in the kernel parameters, so a launch needs no host-to-device copy
// and can be captured in a CUDA graph.
constexpr int kMaxBatchProblems = 224;

struct XProblem {
    const uint8_t *exec;        // execution layout of the packed matrix
    const int64_t *exec_offs;   // units + 1 block offsets in slot order (exec_slot)
    const float *scales;        // per-row-panel F16 scales (else null)
    const void *B;
    void *C;
    int64_t ldb, ldc, M;
    int64_t col_begin;          // first column of the problem's strips
    int64_t col_end;            // columns >= col_end are not computed (NV = 1 tails)
    int64_t item_begin;         // first global item
    int32_t P, S, T, ppt;       // row panels, strips, K tiles, panels per row tile
    int32_t load_c, epilogue;
    const int32_t *panel_rank;  // panel -> position in the work order (exec_slot)
    int32_t order;              // job order: 0 = row panels outer (a panel's strips in a row), 1 = strips outer
    int32_t pad_;
};
static_assert(sizeof(XProblem) == 128, "XProblem layout");

struct BatchParams {
    int *counter;               // work counter, zero at launch
    int *status;                // device status word of bounded waits
    int64_t items;              // total items
    int32_t nprob, xbuf;        // problems; bytes of one per-warp buffer
    XProblem prob[kMaxBatchProblems];
};

struct XJob {
    int64_t gp;   // row panel
    int32_t pi;   // problem index (-1: no job)
    int32_t strip, t;
};

__device__ __forceinline__ int find_problem(const BatchParams &bp, int64_t item) {
    int lo = 0, hi = bp.nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bp.prob[mid].item_begin <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Next job after `j` in this warp's sequence: the next K tile of the same item, or a new item.
__device__ __forceinline__ XJob next_job(const BatchParams &bp, const XJob &j, int *counter, int lane) {
    if (j.pi >= 0 && j.t + 1 < bp.prob[j.pi].T) return XJob{j.gp, j.pi, j.strip, j.t + 1};
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    const int64_t item = __shfl_sync(0xffffffffu, it, 0);
    if (item >= bp.items) return XJob{0, -1, 0, 0};
    const int pi = find_problem(bp, item);
    const XProblem &pr = bp.prob[pi];
    const int64_t local = item - pr.item_begin;
    if (pr.order == 1) return XJob{local % pr.P, pi, (int32_t)(local / pr.P), 0};
    return XJob{local / pr.S, pi, (int32_t)(local % pr.S), 0};
}

__device__ __forceinline__ void issue_job(const BatchParams &bp, const XJob &j, uint32_t buf, uint32_t bar, int lane) {
    if (lane == 0 && j.pi >= 0) {
        const XProblem &pr = bp.prob[j.pi];
        const int64_t slot = exec_slot(j.gp, j.t, pr.P, pr.panel_rank);
        const int64_t off = pr.exec_offs[slot];
        const uint32_t bytes = (uint32_t)(pr.exec_offs[slot + 1] - off);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, bytes);
        bulk_copy_g2s(buf, pr.exec + off, bytes, bar);
    }
}

// C tile init / store for one (problem, panel, strip).
template <int MR, int NV, class TV, class TC, class IO = VecIO<NV, TC>>
__device__ __forceinline__ void x_acc_init(const XProblem &pr, int64_t row0, int64_t col0, bool valid,
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
            if (row0 + r < pr.M) IO::load_plain(C + (row0 + r) * pr.ldc + col0, acc[r]);
    }
}
template <int MR, int NV, class TV, class TC, class IO = VecIO<NV, TC>>
__device__ __forceinline__ void x_store(const XProblem &pr, int64_t gp, int64_t row0, int64_t col0, bool valid,
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
                IO::load_plain(cp, cin);
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
        IO::store(cp, o);
    }
}

// Wide FP32 strips run CTAs of at most 4 warps (kWideMaxWarps).  Their 64-register B step and up
// to 64 accumulators leave 8 warps an SM; where 168 registers a thread suffice without more than a
// few spilled bytes (256 columns, and 512 at M_r <= 2) they are held to that: 3 CTAs, 12 warps.
constexpr int kWideMaxWarps = 4;
template <int MR, int NV, class TB> constexpr int batch_max_threads() {
    return NV >= 8 && sizeof(TB) == 4 ? 32 * kWideMaxWarps : 256;
}
template <int MR, int NV, class TB> constexpr int batch_min_blocks() {
    return NV >= 8 && sizeof(TB) == 4 && (NV == 8 || MR <= 2) ? 3 : 1;
}

template <int MR, int NV, class TV, class TB, class TC>
__global__ void __launch_bounds__(batch_max_threads<MR, NV, TB>(), batch_min_blocks<MR, NV, TB>())
    exec_batch_kernel(const __grid_constant__ BatchParams bp) {
    // NV = 8 and 16 with FP32: strips of 256 and 512 columns in the interleaved lane layout
    // (WideIO).  16-bit B: NV = 8, 256 columns, 8 contiguous a lane (one 16-byte load); NV = 16,
    // 512 columns, 8 a lane in each 256-column half (HalvesIO).
    constexpr bool WIDE = NV >= 8 && sizeof(TB) == 4;
    static_assert(!WIDE || (sizeof(TV) == 4 && sizeof(TC) == 4), "wide FP32 gather strips are FP32 values, B and C");
    static_assert(NV <= 4 || WIDE || ((NV == 8 || NV == 16) && MR <= 4), "16-bit gather strips: NV 8 / 16 at M_r <= 4");
    constexpr int LANE_COLS = WIDE ? 4 : (NV == 16 ? 8 : NV);
    using IO = std::conditional_t<WIDE, WideIO<NV>, std::conditional_t<(NV == 16), HalvesIO<NV, TC>, VecIO<NV, TC>>>;
    using BL = std::conditional_t<WIDE, GlobalBWide<NV>, GlobalB<NV, TB>>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t bar0 = sbase + 16u * warp, bar1 = bar0 + 8u;
    const uint32_t xb = (uint32_t)bp.xbuf;
    const uint32_t buf0 = sbase + 1024u + 2u * xb * warp, buf1 = buf0 + xb;
    if (lane == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar1, 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async_smem();
    __syncwarp();

    XJob j0 = next_job(bp, XJob{0, -1, 0, 0}, bp.counter, lane);
    issue_job(bp, j0, buf0, bar0, lane);
    XJob j1 = next_job(bp, j0, bp.counter, lane);
    issue_job(bp, j1, buf1, bar1, lane);
    XJob last = j1;
    uint32_t ph0 = 0u, ph1 = 0u;
    float acc[MR][NV];

#pragma unroll 1
    for (int b = 0;; b ^= 1) {
        const XJob j = b ? j1 : j0;
        if (j.pi < 0) break;
        const uint32_t buf = b ? buf1 : buf0, bar = b ? bar1 : bar0;
        if (!mbar_wait_bounded(bar, b ? ph1 : ph0, bp.status, 2)) break;
        if (b) ph1 ^= 1u; else ph0 ^= 1u;
        const XProblem &pr = bp.prob[j.pi];
        const int64_t row0 = j.gp * MR;
        const int64_t col0 = pr.col_begin + (int64_t)j.strip * (32 * NV) + (int64_t)lane * LANE_COLS;
        const bool valid = col0 < pr.col_end;
        if (j.t == 0) x_acc_init<MR, NV, TV, TC, IO>(pr, row0, col0, valid, acc);
        const BL bl{reinterpret_cast<const TB *>(pr.B) + col0, pr.ldb, valid};
        const uint32_t G = lds_u32(buf);
#pragma unroll 1
        for (uint32_t g = 0; g < G; ++g) {
            const uint4 rec = lds_u128(buf + 16u + 16u * g);
            run_group_x<MR, NV, TV>((int)rec.x, (int)rec.y, buf + rec.z, buf + rec.w, bl, acc);
        }
        __syncwarp();
        // refill this buffer with the job after the last one issued
        const XJob jn = next_job(bp, last, bp.counter, lane);
        issue_job(bp, jn, buf, bar, lane);
        last = jn;
        if (b) j1 = jn; else j0 = jn;
        if (j.t == pr.T - 1) x_store<MR, NV, TV, TC, IO>(pr, j.gp, row0, col0, valid, acc);
    }
}

// Launch one executor kernel.  One translation unit per (M_r, dtype combination) instantiates
// launch_exec (generated by build.py) so that the kernels compile in parallel.
enum ExecCombo { COMBO_F32 = 0, COMBO_BF16_F32OUT = 1, COMBO_BF16_BF16OUT = 2, COMBO_F16_F32OUT = 3, NUM_COMBOS = 4 };

template <int COMBO> struct ComboTypes;
template <> struct ComboTypes<COMBO_F32> { using V = float; using B = float; using C = float; };
template <> struct ComboTypes<COMBO_BF16_F32OUT> { using V = __nv_bfloat16; using B = __nv_bfloat16; using C = float; };
template <> struct ComboTypes<COMBO_BF16_BF16OUT> { using V = __nv_bfloat16; using B = __nv_bfloat16; using C = __nv_bfloat16; };
template <> struct ComboTypes<COMBO_F16_F32OUT> { using V = __half; using B = __half; using C = float; };

// Largest dynamic shared memory a staged-strip CTA may use (opt-in limit of sm_100-class parts).
constexpr int kMaxSmem = 227 * 1024;

// Wide strips of the gather kernel: FP32 256 (NV = 8) and 512 columns (NV = 16, M_r <= 4); 16-bit
// B 256 and 512 columns (NV = 8, 16; M_r <= 4).
using BatchKernelPtr = void (*)(BatchParams);
template <int MR, int NV, class V, class B, class C> inline BatchKernelPtr wide_batch_kernel() {
    if constexpr (sizeof(V) == 4 && sizeof(B) == 4 && sizeof(C) == 4 && (NV == 8 || MR <= 4))
        return exec_batch_kernel<MR, NV, V, B, C>;
    else if constexpr (sizeof(B) == 2 && (NV == 8 || NV == 16) && MR <= 4)
        return exec_batch_kernel<MR, NV, V, B, C>;
    else
        return nullptr;
}

template <int MR, int COMBO>
cudaError_t launch_exec(const ExecParams &p, int nv, dim3 grid, int threads, cudaStream_t s);
template <int MR, int COMBO>
cudaError_t launch_exec_batch(const BatchParams &p, int nv, unsigned grid, int threads, size_t smem, cudaStream_t s);

#define SPREG_INSTANTIATE_EXEC(MR, COMBO)                                                             \
    template <>                                                                                       \
    cudaError_t launch_exec<MR, COMBO>(const ExecParams &p, int nv, dim3 grid, int threads, cudaStream_t s) { \
        using V = ComboTypes<COMBO>::V;                                                               \
        using B = ComboTypes<COMBO>::B;                                                               \
        using C = ComboTypes<COMBO>::C;                                                               \
        switch (nv) {                                                                                 \
        case 1: exec_kernel<MR, 1, V, B, C><<<grid, threads, 0, s>>>(p); break;                       \
        case 2: exec_kernel<MR, 2, V, B, C><<<grid, threads, 0, s>>>(p); break;                       \
        case 4: exec_kernel<MR, 4, V, B, C><<<grid, threads, 0, s>>>(p); break;                       \
        default: return cudaErrorInvalidValue;                                                        \
        }                                                                                             \
        return cudaGetLastError();                                                                    \
    }                                                                                                 \
    template <>                                                                                       \
    cudaError_t launch_exec_batch<MR, COMBO>(const BatchParams &p, int nv, unsigned grid, int threads, size_t smem, \
                                             cudaStream_t s) {                                        \
        using V = ComboTypes<COMBO>::V;                                                               \
        using B = ComboTypes<COMBO>::B;                                                               \
        using C = ComboTypes<COMBO>::C;                                                               \
        static std::atomic<bool> configured[64][17];                                                          \
        int dev = 0;                                                                                  \
        cudaGetDevice(&dev);                                                                          \
        auto run = [&](auto kern) -> cudaError_t {                                                    \
            if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;                                  \
            if (!configured[dev][nv].load()) {                                                               \
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem); \
                if (e != cudaSuccess) return e;                                                       \
                configured[dev][nv].store(true);                                                           \
            }                                                                                         \
            /* at most the CTAs that can be resident at once (registers included): later ones would */ \
            /* only start once the work list is empty, and then exit */                               \
            int occ = 0, nsm = 0;                                                                     \
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem) == cudaSuccess && occ > 0 && \
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && nsm > 0) \
                grid = std::min<unsigned>(grid, (unsigned)occ * (unsigned)nsm);                       \
            kern<<<grid, threads, smem, s>>>(p);                                                      \
            return cudaGetLastError();                                                                \
        };                                                                                            \
        switch (nv) {                                                                                 \
        case 1: return run(exec_batch_kernel<MR, 1, V, B, C>);                                        \
        case 2: return run(exec_batch_kernel<MR, 2, V, B, C>);                                        \
        case 4: return run(exec_batch_kernel<MR, 4, V, B, C>);                                        \
        case 8: {                                                                                     \
            auto k8 = wide_batch_kernel<MR, 8, V, B, C>();                                            \
            return k8 ? run(k8) : cudaErrorInvalidValue;                                              \
        }                                                                                             \
        case 16: {                                                                                    \
            auto k16 = wide_batch_kernel<MR, 16, V, B, C>();                                          \
            return k16 ? run(k16) : cudaErrorInvalidValue;                                            \
        }                                                                                             \
        default: return cudaErrorInvalidValue;                                                        \
        }                                                                                             \
    }

}  // namespace spreg
