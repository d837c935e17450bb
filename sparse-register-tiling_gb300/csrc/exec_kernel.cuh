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

// ------------------------------------------------------------------ nanokernel loops
// acc[r] += value * b for every set row r of PAT, values consumed in ascending row order.
template <int PAT, int MR, int NV, class TV>
__device__ __forceinline__ void fma_pattern(const TV *__restrict__ v, const float (&b)[NV], float (&acc)[MR][NV]) {
    int q = 0;
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        if ((PAT >> r) & 1) {
            const float a = DT<TV>::to_f32(__ldg(v + q));
            ++q;
#pragma unroll
            for (int j = 0; j < NV; ++j) acc[r][j] = fmaf(a, b[j], acc[r][j]);
        }
    }
}

// n entries of one nanokernel id.  NV == 1 lanes may lie past the last column (valid == false):
// they read zeros and never store.  NV > 1 launches only cover whole strips.
template <int PAT, int MR, int NV, class TV, class TB>
__device__ __forceinline__ void run_group(const int n, const int32_t *__restrict__ cols, const TV *__restrict__ vals,
                                          const TB *__restrict__ Bc, const int64_t ldb, const bool valid,
                                          float (&acc)[MR][NV]) {
    constexpr int PC = cpopc(PAT);
#pragma unroll 2
    for (int e = 0; e < n; ++e) {
        const int64_t k = __ldg(cols + e);
        float b[NV];
        if constexpr (NV == 1) {
            b[0] = valid ? DT<TB>::to_f32(__ldg(Bc + k * ldb)) : 0.0f;
        } else {
            VecIO<NV, TB>::load(Bc + k * ldb, b);
        }
        fma_pattern<PAT, MR, NV, TV>(vals + e * PC, b, acc);
    }
}

// M_r = 8 has 255 patterns; compiling a loop per pattern takes minutes, so M_r = 8 specialises the
// single rows and the nanokernels of the reference's M_r = 8 "orig" (400fa) and "alt" (747f9) sets
// (tools/paper/configs.py:84-87) and runs any other pattern through run_group_nibbles.
template <int MR>
__host__ __device__ constexpr bool fast_pattern(int P) {
    if (P <= 0 || P >= (1 << MR)) return false;
    if (MR < 8) return true;
    switch (P) {
    case 1: case 2: case 4: case 8: case 16: case 32: case 64: case 128:
    case 15: case 60: case 85: case 170: case 195: case 240:
    case 63: case 207: case 243: case 252: case 255:
        return true;
    default:
        return false;
    }
}

// Rows BASE .. BASE+3 of a 4-bit sub-pattern Q, values in ascending row order.
template <int Q, int BASE, int MR, int NV, class TV>
__device__ __forceinline__ void fma_nibble(const TV *__restrict__ v, const float (&b)[NV], float (&acc)[MR][NV]) {
    int q = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if ((Q >> r) & 1) {
            const float a = DT<TV>::to_f32(__ldg(v + q));
            ++q;
#pragma unroll
            for (int j = 0; j < NV; ++j) acc[BASE + r][j] = fmaf(a, b[j], acc[BASE + r][j]);
        }
    }
}

// Any M_r = 8 pattern: rows 0-3 then rows 4-7, each through a 16-way switch per entry.
template <int MR, int NV, class TV, class TB>
__device__ __forceinline__ void run_group_nibbles(const int pat, const int n, const int32_t *__restrict__ cols,
                                               const TV *__restrict__ vals, const TB *__restrict__ Bc,
                                               const int64_t ldb, const bool valid, float (&acc)[MR][NV]) {
    if constexpr (MR == 8) {
        const int lo = pat & 15, hi = (pat >> 4) & 15;
        const int plo = __popc(lo), pc = __popc(pat);
        for (int e = 0; e < n; ++e) {
            const int64_t k = __ldg(cols + e);
            float b[NV];
            if constexpr (NV == 1) {
                b[0] = valid ? DT<TB>::to_f32(__ldg(Bc + k * ldb)) : 0.0f;
            } else {
                VecIO<NV, TB>::load(Bc + k * ldb, b);
            }
            const TV *v = vals + (int64_t)e * pc;
#define SPREG_NIB_LO(Q) case Q: fma_nibble<Q, 0, MR, NV, TV>(v, b, acc); break;
#define SPREG_NIB_HI(Q) case Q: fma_nibble<Q, 4, MR, NV, TV>(v + plo, b, acc); break;
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
        }
    }
}

#define SPREG_C4(F, b) F((b)) F((b) + 1) F((b) + 2) F((b) + 3)
#define SPREG_C16(F, b) SPREG_C4(F, b) SPREG_C4(F, (b) + 4) SPREG_C4(F, (b) + 8) SPREG_C4(F, (b) + 12)
#define SPREG_C64(F, b) SPREG_C16(F, b) SPREG_C16(F, (b) + 16) SPREG_C16(F, (b) + 32) SPREG_C16(F, (b) + 48)

template <int MR, int NV, class TV, class TB>
__device__ __forceinline__ void dispatch_group(const int pat, const int n, const int32_t *__restrict__ cols,
                                               const TV *__restrict__ vals, const TB *__restrict__ Bc,
                                               const int64_t ldb, const bool valid, float (&acc)[MR][NV]) {
#define SPREG_CASE(P)                                                                                 \
    case (P):                                                                                         \
        if constexpr (fast_pattern<MR>(P)) {                                                          \
            run_group<fast_pattern<MR>(P) ? (P) : 1, MR, NV, TV, TB>(n, cols, vals, Bc, ldb, valid, acc); \
            return;                                                                                   \
        }                                                                                             \
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
    if constexpr (MR == 8) run_group_nibbles<MR, NV, TV, TB>(pat, n, cols, vals, Bc, ldb, valid, acc);
}

// ------------------------------------------------------------------ the kernel
template <int MR, int NV, class TV, class TB, class TC>
__global__ void __launch_bounds__(256) exec_kernel(const __grid_constant__ ExecParams p) {
    const int lane = threadIdx.x & 31;
    const int64_t gp = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gp >= p.P) return;
    const int64_t col0 = p.col_begin + (int64_t)blockIdx.y * (32 * NV) + (int64_t)lane * NV;
    const bool valid = col0 < p.N;  // NV > 1 launches cover whole strips only
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

    const TB *Bc = reinterpret_cast<const TB *>(p.B) + col0;
    for (int64_t tj = 0; tj < p.T; ++tj) {
        const spreg_panel_desc d = p.descs[unit_index(gp, tj, p.ppt, p.T, p.P)];
        if (d.num_cols == 0) continue;
        const int32_t *__restrict__ cnt = reinterpret_cast<const int32_t *>(p.arena + d.counts_off);
        const int32_t *__restrict__ cols = reinterpret_cast<const int32_t *>(p.arena + d.cols_off);
        const TV *__restrict__ vals = reinterpret_cast<const TV *>(p.arena + d.values_off);
        for (int id = 0; id < p.nk; ++id) {
            const int n = __ldg(cnt + id);
            if (n == 0) continue;
            const int pat = p.id_pattern[id];
            dispatch_group<MR, NV, TV, TB>(pat, n, cols, vals, Bc, p.ldb, valid, acc);
            cols += n;
            vals += n * __popc(pat);
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

// Launch one executor kernel.  One translation unit per (M_r, dtype combination) instantiates
// launch_exec (generated by build.py) so that the kernels compile in parallel.
enum ExecCombo { COMBO_F32 = 0, COMBO_BF16_F32OUT = 1, COMBO_BF16_BF16OUT = 2, COMBO_F16_F32OUT = 3, NUM_COMBOS = 4 };

template <int COMBO> struct ComboTypes;
template <> struct ComboTypes<COMBO_F32> { using V = float; using B = float; using C = float; };
template <> struct ComboTypes<COMBO_BF16_F32OUT> { using V = __nv_bfloat16; using B = __nv_bfloat16; using C = float; };
template <> struct ComboTypes<COMBO_BF16_BF16OUT> { using V = __nv_bfloat16; using B = __nv_bfloat16; using C = __nv_bfloat16; };
template <> struct ComboTypes<COMBO_F16_F32OUT> { using V = __half; using B = __half; using C = float; };

template <int MR, int COMBO>
cudaError_t launch_exec(const ExecParams &p, int nv, dim3 grid, int threads, cudaStream_t s);

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
        case 8: exec_kernel<MR, 8, V, B, C><<<grid, threads, 0, s>>>(p); break;                       \
        default: return cudaErrorInvalidValue;                                                        \
        }                                                                                             \
        return cudaGetLastError();                                                                    \
    }

}  // namespace spreg
