// pack.cu -- GPU MicroKernelPacker: integer kernels that turn a sparse A into the packed
// sparse-register-tiling arena, byte for byte the layout of SOPTile::pack_panel/pack_tile
// (sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:129-261).
//
// One CTA owns one packed unit (an M_r-row panel, or one panel of an M_c x K_c tile).
//   count pass : pattern of every column (bit r = row r nonzero, sop_utils.py:25-30), the
//                mapping's code list (sop_driver.py:50-65), per-id entry counts, values,
//                padding zeros and the invariant num_nnz == padding + nnz (template:214).
//   layout pass: one CTA scans unit sizes into 64-byte-aligned arena offsets (template:222-258).
//   emit pass  : the stable sort by nanokernel id with the zero pattern dropped (template:70-98,
//                148-158) is a counting sort: per chunk of 256 slots each id keeps a 256-bit
//                bitmap of the slots that carry it, so a slot's rank inside its id is a prefix
//                popcount.  Values of an entry are written in ascending row order (template:192-207).
#include "spreg_common.cuh"

#include <algorithm>
#include <vector>

namespace spreg {

constexpr int CH = 256;        // slots per chunk == threads per packer CTA
constexpr int CHW = CH / 32;   // bitmap words per id per chunk

// ------------------------------------------------------------------ column sources
// A loader fills s_val[r][c] (r < mr, c < w) with A[row0 + r][c0 + c] (zero beyond M) and ends
// with __syncthreads().  The caller must have synchronised since the last read of s_val.
struct DenseLoader {
    const float *A;
    int64_t lda;
    int64_t M;
    __device__ void load(float (*s_val)[CH], uint32_t (*)[CHW], int64_t row0, int mr, int64_t c0, int w,
                         DevError *, int64_t) const {
        const int t = threadIdx.x;
        for (int r = 0; r < mr; ++r) {
            const int64_t row = row0 + r;
            float v = 0.0f;
            if (t < w && row < M) v = A[row * lda + c0 + t];
            s_val[r][t] = v;
        }
        __syncthreads();
    }
};

struct CsrLoader {
    const int32_t *row_ptrs;
    const int32_t *col_inds;
    const float *values;
    int64_t M;
    __device__ void load(float (*s_val)[CH], uint32_t (*s_seen)[CHW], int64_t row0, int mr, int64_t c0, int w,
                         DevError *err, int64_t unit) const {
        const int t = threadIdx.x;
        for (int r = 0; r < mr; ++r) s_val[r][t] = 0.0f;
        if (t < mr * CHW) s_seen[t / CHW][t % CHW] = 0u;
        __syncthreads();
        for (int r = 0; r < mr; ++r) {
            const int64_t row = row0 + r;
            if (row >= M) break;
            const int32_t beg = row_ptrs[row], end = row_ptrs[row + 1];
            for (int32_t p = beg + t; p < end; p += CH) {
                const int64_t col = col_inds[p];
                if (col >= c0 && col < c0 + w) {
                    const int lc = (int)(col - c0);
                    const uint32_t bit = 1u << (lc & 31);
                    const uint32_t old = atomicOr(&s_seen[r][lc >> 5], bit);
                    if ((old & bit) && err) {
                        if (atomicCAS(&err->code, 0, 3) == 0) { err->unit = (int32_t)unit; err->value = (int32_t)col; }
                    }
                    s_val[r][lc] = values[p];
                }
            }
        }
        __syncthreads();
    }
};

__device__ inline void raise_err(DevError *err, int code, int64_t unit, int value) {
    if (atomicCAS(&err->code, 0, code) == 0) {
        err->unit = (int32_t)unit;
        err->value = value;
    }
}

__device__ inline void load_map_table(MapTable *s_mt, const MapTable *g) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g);
    uint32_t *dst = reinterpret_cast<uint32_t *>(s_mt);
    for (int i = threadIdx.x; i < (int)(sizeof(MapTable) / 4); i += blockDim.x) dst[i] = src[i];
}

// Block-wide sum of an int over 256 threads.
__device__ inline long long block_sum(long long v, long long *s_tmp) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) s_tmp[warp] = v;
    __syncthreads();
    long long tot = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) tot += s_tmp[i];
    return tot;  // valid on thread 0
}

__device__ inline float block_max(float v, float *s_tmp) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) s_tmp[warp] = v;
    __syncthreads();
    float m = 0.0f;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmaxf(m, s_tmp[i]);
    return m;
}

// Execution block size of a unit from its per-id counts (thread 0 of the CTA).
__device__ inline void exec_size(const MapTable &mt, const int *counts, int vb, int32_t *bytes, int32_t *groups) {
    int64_t sz = sizeof(ExecHeader);
    int g = 0;
    for (int id = 0; id < mt.num_nkern; ++id) {
        const int64_t n = counts[id];
        if (!n) continue;
        ++g;
        sz += sizeof(ExecGroup) + exec_cols_bytes(n) + exec_vals_bytes(n, __popc(mt.id_to_pattern[id]), vb);
    }
    *bytes = (int32_t)sz;
    *groups = g;
}

// ------------------------------------------------------------------ count pass (columns)
template <class Loader>
__global__ void __launch_bounds__(CH) count_cols_kernel(const Geom g, const Loader ld, const MapTable *__restrict__ mt,
                                                        int32_t *__restrict__ unit_counts, UnitStats *__restrict__ stats,
                                                        unsigned *__restrict__ panel_maxabs,
                                                        unsigned long long *__restrict__ tile_nnz, DevError *err,
                                                        const int vb) {
    __shared__ MapTable s_mt;
    __shared__ float s_val[SPREG_MAX_MR][CH];
    __shared__ uint32_t s_seen[SPREG_MAX_MR][CHW];
    __shared__ int s_count[256];
    __shared__ long long s_tmp[CH / 32];
    __shared__ float s_ftmp[CH / 32];

    const int64_t u = blockIdx.x;
    int64_t gp, tj;
    unit_coords(u, g.ppt, g.T, g.P, &gp, &tj);
    const int64_t c_lo = tj * g.kt;
    const int64_t c_hi = (c_lo + g.kt < g.K) ? c_lo + g.kt : g.K;

    load_map_table(&s_mt, mt);
    for (int i = threadIdx.x; i < 256; i += CH) s_count[i] = 0;
    __syncthreads();
    const int mr = s_mt.mr;

    long long nnz = 0, nv = 0, pad = 0;
    float mx = 0.0f;
    for (int64_t c0 = c_lo; c0 < c_hi; c0 += CH) {
        const int w = (int)((c_hi - c0) < CH ? (c_hi - c0) : CH);
        ld.load(s_val, s_seen, gp * mr, mr, c0, w, err, u);
        const int t = threadIdx.x;
        if (t < w) {
            int pat = 0;
            for (int r = 0; r < mr; ++r) {
                const float v = s_val[r][t];
                if (v != 0.0f) pat |= 1 << r;
                mx = fmaxf(mx, fabsf(v));
            }
            nnz += __popc(pat);
            const int ncodes = s_mt.map_n[pat];
            for (int q = 0; q < ncodes; ++q) {
                const int code = s_mt.map_codes[pat][q];
                const int id = s_mt.code_to_id[code];
                if (id >= s_mt.num_nkern) { raise_err(err, 1, u, code); continue; }
                atomicAdd(&s_count[id], 1);
                nv += __popc(code);
                pad += __popc(code & ~pat);
            }
        }
        __syncthreads();
    }
    const long long tot_nnz = block_sum(nnz, s_tmp);
    const long long tot_v = block_sum(nv, s_tmp);
    const long long tot_pad = block_sum(pad, s_tmp);
    const float tot_mx = block_max(mx, s_ftmp);
    const int nk = s_mt.num_nkern;
    for (int id = threadIdx.x; id < nk; id += CH) unit_counts[u * nk + id] = s_count[id];
    if (threadIdx.x == 0) {
        long long nu = 0;
        for (int id = 0; id < nk; ++id) nu += s_count[id];
        int32_t xb, xg;
        exec_size(s_mt, s_count, vb, &xb, &xg);
        stats[u] = UnitStats{(int32_t)nu, (int32_t)tot_v, (int32_t)tot_pad, (int32_t)tot_nnz, xb, xg};
        if (tot_v != tot_pad + tot_nnz) raise_err(err, 2, u, (int)tot_v);
        atomicMax(&panel_maxabs[gp], __float_as_uint(tot_mx));
        const int64_t ti = gp / g.ppt;
        atomicAdd(&tile_nnz[ti * g.T + tj], (unsigned long long)tot_nnz);
    }
}

// ------------------------------------------------------------------ count pass (entry lists)
// SOPTile path: panel p has entries [entry_off[p], entry_off[p+1]) of (code, column) in caller
// order and a dense (panel_cols[p] x mr) block at dense + dense_off[p].
struct ListSrc {
    const int32_t *codes;
    const int32_t *cols;
    const int64_t *entry_off;
    const float *dense;
    const int64_t *dense_off;
    const int64_t *panel_cols;
    const int64_t *col_offset;
};

__global__ void __launch_bounds__(CH) count_list_kernel(const ListSrc src, const MapTable *__restrict__ mt,
                                                        int32_t *__restrict__ unit_counts,
                                                        UnitStats *__restrict__ stats, unsigned *__restrict__ panel_maxabs,
                                                        unsigned long long *__restrict__ tile_nnz, DevError *err,
                                                        const int vb) {
    __shared__ MapTable s_mt;
    __shared__ int s_count[256];
    __shared__ long long s_tmp[CH / 32];
    __shared__ float s_ftmp[CH / 32];
    const int64_t p = blockIdx.x;
    load_map_table(&s_mt, mt);
    for (int i = threadIdx.x; i < 256; i += CH) s_count[i] = 0;
    __syncthreads();
    const int mr = s_mt.mr;
    const float *dense = src.dense + src.dense_off[p];
    const int64_t K = src.panel_cols[p];
    long long nnz = 0, nv = 0, pad = 0;
    float mx = 0.0f;
    for (int64_t i = threadIdx.x; i < K * mr; i += CH) {
        const float v = dense[i];
        nnz += v != 0.0f;
        mx = fmaxf(mx, fabsf(v));
    }
    for (int64_t e = src.entry_off[p] + threadIdx.x; e < src.entry_off[p + 1]; e += CH) {
        const int code = src.codes[e];
        const int64_t col = src.cols[e];
        const int id = (code >= 0 && code < 256) ? (int)s_mt.code_to_id[code] : (int)kCodeInvalid;
        if (id == kCodeZero) continue;
        if (id >= s_mt.num_nkern) { raise_err(err, 1, p, code); continue; }
        if (col < 0 || col >= K) { raise_err(err, 4, p, (int)col); continue; }
        atomicAdd(&s_count[id], 1);
        nv += __popc(code);
        for (int r = 0; r < mr; ++r)
            if ((code >> r) & 1) pad += dense[col * mr + r] == 0.0f;
    }
    __syncthreads();
    const long long tot_nnz = block_sum(nnz, s_tmp);
    const long long tot_v = block_sum(nv, s_tmp);
    const long long tot_pad = block_sum(pad, s_tmp);
    const float tot_mx = block_max(mx, s_ftmp);
    const int nk = s_mt.num_nkern;
    for (int id = threadIdx.x; id < nk; id += CH) unit_counts[p * nk + id] = s_count[id];
    if (threadIdx.x == 0) {
        long long nu = 0;
        for (int id = 0; id < nk; ++id) nu += s_count[id];
        int32_t xb, xg;
        exec_size(s_mt, s_count, vb, &xb, &xg);
        stats[p] = UnitStats{(int32_t)nu, (int32_t)tot_v, (int32_t)tot_pad, (int32_t)tot_nnz, xb, xg};
        if (tot_v != tot_pad + tot_nnz) raise_err(err, 2, p, (int)tot_v);
        panel_maxabs[p] = __float_as_uint(tot_mx);
        atomicAdd(&tile_nnz[0], (unsigned long long)tot_nnz);
    }
}

// ------------------------------------------------------------------ layout pass
// Inclusive prefix sum of one value per thread of a 1024-thread block (shuffles within warps, one
// warp over the 32 warp totals); *total = the block's sum.  s_warp holds 32 entries.
__device__ __forceinline__ long long block_incl_scan(long long v, long long *s_warp, long long *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) s_warp[w] = v;
    __syncthreads();
    if (w == 0) {
        long long x = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        s_warp[lane] = x;
    }
    __syncthreads();
    if (w > 0) v += s_warp[w - 1];
    *total = s_warp[31];
    __syncthreads();  // s_warp is reused by the next call
    return v;
}

__global__ void __launch_bounds__(1024) layout_kernel(const int64_t units, const int nk, const int vb,
                                                      const int64_t ppt, const int64_t T, const int64_t P,
                                                      const UnitStats *__restrict__ stats,
                                                      const unsigned long long *__restrict__ tile_nnz,
                                                      spreg_panel_desc *__restrict__ descs, PackTotals *tot) {
    __shared__ long long s_warp[32];
    __shared__ unsigned long long s_acc[8];
    const int t = threadIdx.x;
    if (t < 8) s_acc[t] = 0;
    __syncthreads();
    long long carry = 0, xtotal = 0;
    long long my_v = 0, my_u = 0, my_pad = 0, my_nnz = 0, my_req = 0, my_empty = 0, my_xmax = 0;
    for (int64_t base = 0; base < units; base += 1024) {
        const int64_t u = base + t;
        long long size = 0;
        UnitStats st = {0, 0, 0, 0, 0, 0};
        if (u < units) {
            st = stats[u];
            const long long xsize = st.exec_bytes;
            xtotal += xsize;
            my_xmax = xsize > my_xmax ? xsize : my_xmax;
            size = align64((int64_t)st.num_values * vb) + align64((int64_t)st.num_cols * 4) + align64((int64_t)nk * 4);
            my_v += st.num_values;
            my_u += st.num_cols;
            my_pad += st.padding;
            my_nnz += st.nnz;
            my_req += (long long)st.num_values * vb + (long long)st.num_cols * 4 + (long long)nk * 4 + 3 * 64;
            int64_t gp, tj;
            unit_coords(u, ppt, T, P, &gp, &tj);
            if (tile_nnz[(gp / ppt) * T + tj] == 0) my_empty++;
        }
        long long chunk = 0;
        const long long incl = block_incl_scan(size, s_warp, &chunk);
        if (u < units) {
            const long long off = carry + incl - size;
            spreg_panel_desc d;
            d.values_off = off;
            d.cols_off = off + align64((int64_t)st.num_values * vb);
            d.counts_off = d.cols_off + align64((int64_t)st.num_cols * 4);
            d.num_values = st.num_values;
            d.num_cols = st.num_cols;
            descs[u] = d;
        }
        carry += chunk;
    }
    long long my_x = xtotal;
    // warp sums first: one shared atomic per warp instead of 1024 contending ones
    for (int o = 16; o > 0; o >>= 1) {
        my_v += __shfl_down_sync(0xffffffffu, my_v, o);
        my_u += __shfl_down_sync(0xffffffffu, my_u, o);
        my_pad += __shfl_down_sync(0xffffffffu, my_pad, o);
        my_nnz += __shfl_down_sync(0xffffffffu, my_nnz, o);
        my_req += __shfl_down_sync(0xffffffffu, my_req, o);
        my_empty += __shfl_down_sync(0xffffffffu, my_empty, o);
        my_x += __shfl_down_sync(0xffffffffu, my_x, o);
        const long long xm = __shfl_down_sync(0xffffffffu, my_xmax, o);
        my_xmax = xm > my_xmax ? xm : my_xmax;
    }
    if ((t & 31) == 0) {
        atomicAdd(&s_acc[0], (unsigned long long)my_v);
        atomicAdd(&s_acc[1], (unsigned long long)my_u);
        atomicAdd(&s_acc[2], (unsigned long long)my_pad);
        atomicAdd(&s_acc[3], (unsigned long long)my_nnz);
        atomicAdd(&s_acc[4], (unsigned long long)my_req);
        atomicAdd(&s_acc[5], (unsigned long long)my_empty);
        atomicAdd(&s_acc[6], (unsigned long long)my_x);
        atomicMax(&s_acc[7], (unsigned long long)my_xmax);
    }
    __syncthreads();
    if (t == 0) {
        tot->arena_bytes = carry;
        tot->num_values = (long long)s_acc[0];
        tot->num_cols = (long long)s_acc[1];
        tot->padding = (long long)s_acc[2];
        tot->nnz = (long long)s_acc[3];
        tot->required_storage = (long long)s_acc[4];
        tot->empty_units = (long long)s_acc[5];
        tot->exec_bytes = (long long)s_acc[6];
        tot->max_exec_bytes = (long long)s_acc[7];
    }
}

// Work estimate of each row panel over its K tiles: the executor's cost per entry (index, B row
// load, loop), per value (FMA) and per nanokernel group (record, dispatch).
__global__ void panel_work_kernel(const int64_t P, const int64_t T, const int64_t ppt,
                                  const UnitStats *__restrict__ stats, int64_t *__restrict__ work) {
    const int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gp >= P) return;
    int64_t w = 0;
    for (int64_t t = 0; t < T; ++t) {
        const UnitStats st = stats[unit_index(gp, t, ppt, T, P)];
        w += 3 * (int64_t)st.num_cols + st.num_values + 8 * (int64_t)st.num_groups;
    }
    work[gp] = w;
}

// Entries of each nanokernel id over all units (block = id).
__global__ void id_totals_kernel(const int32_t *__restrict__ unit_counts, const int64_t units, const int nk,
                                 unsigned long long *__restrict__ totals) {
    __shared__ unsigned long long s_sum[32];
    const int id = blockIdx.x;
    unsigned long long sum = 0;
    for (int64_t u = threadIdx.x; u < units; u += blockDim.x) sum += (unsigned)unit_counts[u * nk + id];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_sum[w];
        totals[id] = t;
    }
}

// Offsets of the execution blocks in slot order (exec_slot): exec_offs[slot] for the executors,
// unit_xoff[unit] for the emit kernels.
__global__ void __launch_bounds__(1024) exec_slots_kernel(const int64_t units, const int64_t P, const int64_t T,
                                                          const int64_t ppt, const int32_t *__restrict__ order,
                                                          const UnitStats *__restrict__ stats,
                                                          int64_t *__restrict__ exec_offs,
                                                          int64_t *__restrict__ unit_xoff) {
    __shared__ long long s_warp[32];
    const int t = threadIdx.x;
    long long carry = 0;
    for (int64_t base = 0; base < units; base += 1024) {
        const int64_t s = base + t;
        int64_t u = -1;
        long long xsize = 0;
        if (s < units) {
            u = unit_index(order[s % P], s / P, ppt, T, P);
            xsize = stats[u].exec_bytes;
        }
        long long chunk = 0;
        const long long incl = block_incl_scan(xsize, s_warp, &chunk);
        if (u >= 0) {
            const long long off = carry + incl - xsize;
            exec_offs[s] = off;
            unit_xoff[u] = off;
        }
        carry += chunk;
    }
    if (t == 0) exec_offs[units] = carry;
}

// Power-of-two F16 scale per row panel: 2^e with max|v| = m * 2^e, m in [0.5, 1); 1 if max is 0.
__global__ void scales_kernel(const int64_t P, const unsigned *__restrict__ panel_maxabs, float *__restrict__ scales) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P) return;
    const float mx = __uint_as_float(panel_maxabs[i]);
    float s = 1.0f;
    if (mx > 0.0f && isfinite(mx)) {
        int e;
        frexpf(mx, &e);
        s = ldexpf(1.0f, e);
    }
    scales[i] = s;
}

// ------------------------------------------------------------------ emit pass helpers
struct EmitShared {
    int start[256];
    int vstart[256];
    int run[256];
    int xcol[256];   // byte offset of an id's cols in the unit's execution block
    int xval[256];   // byte offset of an id's values
    uint32_t bits[256][CHW];
    uint16_t pref[256][CHW];
};

// Per-id exclusive scans of entry and value counts; writes the unit's nkern_counts and the
// header and group records of its execution block.
__device__ inline void emit_prologue(EmitShared &s, const MapTable &mt, const int32_t *counts, int32_t *out_counts,
                                     uint8_t *xblock, int vb) {
    const int nk = mt.num_nkern;
    for (int id = threadIdx.x; id < nk; id += blockDim.x) out_counts[id] = counts[id];
    if (threadIdx.x == 0) {
        int e = 0, v = 0, g = 0;
        for (int id = 0; id < nk; ++id) g += counts[id] != 0;
        int64_t off = sizeof(ExecHeader) + (int64_t)g * sizeof(ExecGroup);
        ExecGroup *grp = reinterpret_cast<ExecGroup *>(xblock + sizeof(ExecHeader));
        g = 0;
        for (int id = 0; id < nk; ++id) {
            const int n = counts[id];
            const int pc = __popc(mt.id_to_pattern[id]);
            s.start[id] = e;
            s.vstart[id] = v;
            e += n;
            v += n * pc;
            s.xcol[id] = (int)off;
            s.xval[id] = (int)(off + exec_cols_bytes(n));
            if (n) {
                grp[g++] = ExecGroup{mt.id_to_pattern[id], (uint32_t)n, (uint32_t)s.xcol[id], (uint32_t)s.xval[id]};
                off += exec_cols_bytes(n) + exec_vals_bytes(n, pc, vb);
            }
        }
        *reinterpret_cast<ExecHeader *>(xblock) = ExecHeader{(uint32_t)g, (uint32_t)off, 0u, 0u};
    }
    for (int id = threadIdx.x; id < 256; id += blockDim.x) s.run[id] = 0;
}

__device__ inline void zero_bits(EmitShared &s, int nb) {
    uint32_t *b = &s.bits[0][0];
    for (int i = threadIdx.x; i < nb * CHW; i += blockDim.x) b[i] = 0u;
}

__device__ inline void bits_prefix(EmitShared &s, int nb) {
    for (int i = threadIdx.x; i < nb * CHW; i += blockDim.x) {
        const int id = i / CHW, wd = i % CHW;
        int sum = 0;
        for (int w2 = 0; w2 < wd; ++w2) sum += __popc(s.bits[id][w2]);
        s.pref[id][wd] = (uint16_t)sum;
    }
}

__device__ inline void bits_advance(EmitShared &s, int nb) {
    for (int id = threadIdx.x; id < nb; id += blockDim.x)
        s.run[id] += s.pref[id][CHW - 1] + __popc(s.bits[id][CHW - 1]);
}

__device__ inline int slot_rank(const EmitShared &s, int id, int slot) {
    const int wd = slot >> 5;
    const uint32_t lt = (slot & 31) ? (0xffffffffu >> (32 - (slot & 31))) : 0u;
    return s.run[id] + s.pref[id][wd] + __popc(s.bits[id][wd] & lt);
}

// ------------------------------------------------------------------ emit pass (columns)
template <class Loader, class TV>
__global__ void __launch_bounds__(CH) emit_cols_kernel(const Geom g, const Loader ld, const MapTable *__restrict__ mt,
                                                       const int32_t *__restrict__ unit_counts,
                                                       const spreg_panel_desc *__restrict__ descs,
                                                       uint8_t *__restrict__ arena, const float *__restrict__ scales,
                                                       const int64_t col_offset, uint8_t *__restrict__ exec,
                                                       const int64_t *__restrict__ exec_offs) {
    __shared__ MapTable s_mt;
    __shared__ float s_val[SPREG_MAX_MR][CH];
    __shared__ uint32_t s_seen[SPREG_MAX_MR][CHW];
    __shared__ EmitShared s;

    const int64_t u = blockIdx.x;
    int64_t gp, tj;
    unit_coords(u, g.ppt, g.T, g.P, &gp, &tj);
    const int64_t c_lo = tj * g.kt;
    const int64_t c_hi = (c_lo + g.kt < g.K) ? c_lo + g.kt : g.K;
    const spreg_panel_desc d = descs[u];

    load_map_table(&s_mt, mt);
    __syncthreads();
    const int nk = s_mt.num_nkern;
    const int mr = s_mt.mr;
    uint8_t *xb = exec + exec_offs[u];
    emit_prologue(s, s_mt, unit_counts + u * nk, reinterpret_cast<int32_t *>(arena + d.counts_off), xb,
                  (int)sizeof(TV));
    int32_t *out_cols = reinterpret_cast<int32_t *>(arena + d.cols_off);
    TV *out_vals = reinterpret_cast<TV *>(arena + d.values_off);
    const float inv = scales ? 1.0f / scales[gp] : 1.0f;  // exact: scales are powers of two
    __syncthreads();

    const int t = threadIdx.x;
    for (int64_t c0 = c_lo; c0 < c_hi; c0 += CH) {
        const int w = (int)((c_hi - c0) < CH ? (c_hi - c0) : CH);
        zero_bits(s, nk);
        ld.load(s_val, s_seen, gp * mr, mr, c0, w, nullptr, u);
        int pat = 0;
        if (t < w) {
            for (int r = 0; r < mr; ++r)
                if (s_val[r][t] != 0.0f) pat |= 1 << r;
            for (int q = 0; q < s_mt.map_n[pat]; ++q) {
                const int id = s_mt.code_to_id[s_mt.map_codes[pat][q]];
                atomicOr(&s.bits[id][t >> 5], 1u << (t & 31));
            }
        }
        __syncthreads();
        bits_prefix(s, nk);
        __syncthreads();
        if (t < w) {
            for (int q = 0; q < s_mt.map_n[pat]; ++q) {
                const int code = s_mt.map_codes[pat][q];
                const int id = s_mt.code_to_id[code];
                const int rank = slot_rank(s, id, t);
                const int32_t colv = (int32_t)(c0 + t + col_offset);
                out_cols[s.start[id] + rank] = colv;
                reinterpret_cast<int32_t *>(xb + s.xcol[id])[rank] = colv;
                TV *xv = reinterpret_cast<TV *>(xb + s.xval[id]) + rank * __popc(code);
                int vo = s.vstart[id] + rank * __popc(code);
                for (int r = 0; r < mr; ++r)
                    if ((code >> r) & 1) {
                        float v = s_val[r][t];
                        if (DT<TV>::id == SPREG_F16) v *= inv;
                        const TV q = DT<TV>::from_f32(v);
                        out_vals[vo++] = q;
                        *xv++ = q;
                    }
            }
        }
        __syncthreads();
        bits_advance(s, nk);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ emit pass (entry lists)
template <class TV>
__global__ void __launch_bounds__(CH) emit_list_kernel(const ListSrc src, const MapTable *__restrict__ mt,
                                                       const int32_t *__restrict__ unit_counts,
                                                       const spreg_panel_desc *__restrict__ descs,
                                                       uint8_t *__restrict__ arena, const float *__restrict__ scales,
                                                       uint8_t *__restrict__ exec, const int64_t *__restrict__ exec_offs) {
    __shared__ MapTable s_mt;
    __shared__ EmitShared s;
    const int64_t p = blockIdx.x;
    const spreg_panel_desc d = descs[p];
    load_map_table(&s_mt, mt);
    __syncthreads();
    const int nk = s_mt.num_nkern;
    const int mr = s_mt.mr;
    uint8_t *xb = exec + exec_offs[p];
    emit_prologue(s, s_mt, unit_counts + p * nk, reinterpret_cast<int32_t *>(arena + d.counts_off), xb,
                  (int)sizeof(TV));
    int32_t *out_cols = reinterpret_cast<int32_t *>(arena + d.cols_off);
    TV *out_vals = reinterpret_cast<TV *>(arena + d.values_off);
    const float inv = scales ? 1.0f / scales[p] : 1.0f;
    const float *dense = src.dense + src.dense_off[p];
    const int64_t coff = src.col_offset[p];
    __syncthreads();

    const int t = threadIdx.x;
    const int64_t e_lo = src.entry_off[p], e_hi = src.entry_off[p + 1];
    for (int64_t e0 = e_lo; e0 < e_hi; e0 += CH) {
        const int w = (int)((e_hi - e0) < CH ? (e_hi - e0) : CH);
        zero_bits(s, nk);
        __syncthreads();
        int code = 0, id = kCodeZero;
        int64_t col = 0;
        if (t < w) {
            code = src.codes[e0 + t];
            col = src.cols[e0 + t];
            id = s_mt.code_to_id[code];
            if (id < nk) atomicOr(&s.bits[id][t >> 5], 1u << (t & 31));
        }
        __syncthreads();
        bits_prefix(s, nk);
        __syncthreads();
        if (t < w && id < nk) {
            const int rank = slot_rank(s, id, t);
            const int32_t colv = (int32_t)(col + coff);
            out_cols[s.start[id] + rank] = colv;
            reinterpret_cast<int32_t *>(xb + s.xcol[id])[rank] = colv;
            TV *xv = reinterpret_cast<TV *>(xb + s.xval[id]) + rank * __popc(code);
            int vo = s.vstart[id] + rank * __popc(code);
            for (int r = 0; r < mr; ++r)
                if ((code >> r) & 1) {
                    float v = dense[col * mr + r];
                    if (DT<TV>::id == SPREG_F16) v *= inv;
                    const TV q = DT<TV>::from_f32(v);
                    out_vals[vo++] = q;
                    *xv++ = q;
                }
        }
        __syncthreads();
        bits_advance(s, nk);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ sort_and_encode
// One CTA; buckets are the nk ids plus the zero pattern (last).  Stable within a bucket.
__global__ void __launch_bounds__(CH) sort_encode_kernel(const MapTable *__restrict__ mt,
                                                         const int32_t *__restrict__ codes, const int64_t n,
                                                         int32_t *__restrict__ encoded, int32_t *__restrict__ order,
                                                         DevError *err) {
    __shared__ MapTable s_mt;
    __shared__ int s_count[257];
    __shared__ int s_start[257];
    __shared__ int s_run[257];
    __shared__ uint32_t s_bits[257][CHW];
    __shared__ uint16_t s_pref[257][CHW];
    load_map_table(&s_mt, mt);
    for (int i = threadIdx.x; i < 257; i += CH) { s_count[i] = 0; s_run[i] = 0; }
    __syncthreads();
    const int nk = s_mt.num_nkern;
    const int nb = nk + 1;
    auto bucket_of = [&](int code) -> int {
        if (code < 0 || code > 255) return -1;
        const int id = s_mt.code_to_id[code];
        if (id == kCodeZero) return nk;
        if (id >= nk) return -1;
        return id;
    };
    for (int64_t i = threadIdx.x; i < n; i += CH) {
        const int b = bucket_of(codes[i]);
        if (b < 0) { raise_err(err, 1, i, codes[i]); continue; }
        atomicAdd(&s_count[b], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int e = 0;
        for (int b = 0; b < nb; ++b) { s_start[b] = e; e += s_count[b]; }
    }
    __syncthreads();
    const int t = threadIdx.x;
    for (int64_t e0 = 0; e0 < n; e0 += CH) {
        const int w = (int)((n - e0) < CH ? (n - e0) : CH);
        for (int i = t; i < nb * CHW; i += CH) (&s_bits[0][0])[i] = 0u;
        __syncthreads();
        int b = -1;
        if (t < w) {
            b = bucket_of(codes[e0 + t]);
            if (b >= 0) atomicOr(&s_bits[b][t >> 5], 1u << (t & 31));
        }
        __syncthreads();
        for (int i = t; i < nb * CHW; i += CH) {
            const int bb = i / CHW, wd = i % CHW;
            int sum = 0;
            for (int w2 = 0; w2 < wd; ++w2) sum += __popc(s_bits[bb][w2]);
            s_pref[bb][wd] = (uint16_t)sum;
        }
        __syncthreads();
        if (t < w && b >= 0) {
            const int wd = t >> 5;
            const uint32_t lt = (t & 31) ? (0xffffffffu >> (32 - (t & 31))) : 0u;
            const int pos = s_start[b] + s_run[b] + s_pref[b][wd] + __popc(s_bits[b][wd] & lt);
            order[pos] = (int32_t)(e0 + t);
            encoded[pos] = (b == nk) ? (int32_t)kCodeZero : b;
        }
        __syncthreads();
        for (int i = t; i < nb; i += CH) s_run[i] += s_pref[i][CHW - 1] + __popc(s_bits[i][CHW - 1]);
        __syncthreads();
    }
}

// ================================================================== host drivers
const MapTable *mapping_device_table(const spreg_mapping *m, int *status);

namespace {


// ------------------------------------------------------------------ packed arena import
// Count pass over an arena read back from a file: each unit's descriptor must address bytes inside
// the arena (4-byte aligned), its nkern_counts must be non-negative and add up to num_cols and, with
// the nanokernels' popcounts, to num_values, and its column indices must lie in its K tile.  Then
// the statistics of the ordinary count pass (padding = zero values, execution block size).
__global__ void __launch_bounds__(CH) arena_count_kernel(const Geom g, const MapTable *__restrict__ mt,
                                                         const uint8_t *__restrict__ arena, const int64_t arena_bytes,
                                                         const spreg_panel_desc *__restrict__ descs, const int vb,
                                                         const int64_t col_offset, int32_t *__restrict__ unit_counts,
                                                         UnitStats *__restrict__ stats,
                                                         unsigned long long *__restrict__ tile_nnz, DevError *err) {
    __shared__ MapTable s_mt;
    __shared__ int s_count[256];
    __shared__ int s_ok;
    __shared__ long long s_tmp[CH / 32];
    const int64_t u = blockIdx.x;
    load_map_table(&s_mt, mt);
    __syncthreads();  // the table is read below by every thread
    const spreg_panel_desc d = descs[u];
    const int nk = s_mt.num_nkern;
    if (threadIdx.x == 0) {
        const bool ok = d.num_values >= 0 && d.num_cols >= 0 && d.values_off >= 0 && d.cols_off >= 0 &&
                        d.counts_off >= 0 && d.values_off % 4 == 0 && d.cols_off % 4 == 0 && d.counts_off % 4 == 0 &&
                        d.values_off + (int64_t)d.num_values * vb <= arena_bytes &&
                        d.cols_off + (int64_t)d.num_cols * 4 <= arena_bytes &&
                        d.counts_off + (int64_t)nk * 4 <= arena_bytes;
        s_ok = ok ? 1 : 0;
        if (!ok) raise_err(err, 5, u, 0);
    }
    __syncthreads();
    if (!s_ok) {
        if (threadIdx.x == 0) stats[u] = UnitStats{0, 0, 0, 0, (int32_t)sizeof(ExecHeader), 0};
        for (int id = threadIdx.x; id < nk; id += CH) unit_counts[u * nk + id] = 0;
        return;
    }
    const int32_t *counts = reinterpret_cast<const int32_t *>(arena + d.counts_off);
    for (int id = threadIdx.x; id < 256; id += CH) s_count[id] = id < nk ? counts[id] : 0;
    __syncthreads();
    int64_t gp, tj;
    unit_coords(u, g.ppt, g.T, g.P, &gp, &tj);
    if (threadIdx.x == 0) {
        long long ents = 0, vals = 0;
        bool neg = false;
        for (int id = 0; id < nk; ++id) {
            neg |= s_count[id] < 0;
            ents += s_count[id];
            vals += (long long)s_count[id] * __popc(s_mt.id_to_pattern[id]);
        }
        s_ok = (!neg && ents == d.num_cols && vals == d.num_values) ? 1 : 0;
        if (!s_ok) raise_err(err, 6, u, (int)ents);
    }
    __syncthreads();
    if (!s_ok) {
        if (threadIdx.x == 0) stats[u] = UnitStats{0, 0, 0, 0, (int32_t)sizeof(ExecHeader), 0};
        for (int id = threadIdx.x; id < nk; id += CH) unit_counts[u * nk + id] = 0;
        return;
    }
    const int64_t lo = col_offset + tj * g.kt;
    const int64_t hi = col_offset + ((tj + 1) * g.kt < g.K ? (tj + 1) * g.kt : g.K);
    const int32_t *cols = reinterpret_cast<const int32_t *>(arena + d.cols_off);
    for (int e = threadIdx.x; e < d.num_cols; e += CH)
        if (cols[e] < lo || cols[e] >= hi) raise_err(err, 7, u, cols[e]);
    long long zeros = 0;
    for (int v = threadIdx.x; v < d.num_values; v += CH) {
        const uint8_t *q = arena + d.values_off + (int64_t)v * vb;
        bool z;
        if (vb == 4) z = (*reinterpret_cast<const uint32_t *>(q) & 0x7FFFFFFFu) == 0u;
        else z = (*reinterpret_cast<const uint16_t *>(q) & 0x7FFFu) == 0u;
        zeros += z ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) zeros += __shfl_down_sync(0xffffffffu, zeros, o);
    if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = zeros;
    __syncthreads();
    for (int id = threadIdx.x; id < nk; id += CH) unit_counts[u * nk + id] = s_count[id];
    if (threadIdx.x == 0) {
        long long pad = 0;
        for (int i = 0; i < CH / 32; ++i) pad += s_tmp[i];
        int32_t xb, xg;
        exec_size(s_mt, s_count, vb, &xb, &xg);
        const long long nnz = d.num_values - pad;
        stats[u] = UnitStats{d.num_cols, d.num_values, (int32_t)pad, (int32_t)nnz, xb, xg};
        atomicAdd(&tile_nnz[(gp / g.ppt) * g.T + tj], (unsigned long long)nnz);
    }
}

// Emit pass of an imported arena: the recomputed descriptor must equal the imported one; the
// unit's values and columns are copied and its execution block is written group by group (the
// arena already holds the entries in nanokernel-id order).
__global__ void __launch_bounds__(CH) arena_emit_kernel(const MapTable *__restrict__ mt,
                                                        const uint8_t *__restrict__ src,
                                                        const spreg_panel_desc *__restrict__ src_descs,
                                                        const int32_t *__restrict__ unit_counts,
                                                        const spreg_panel_desc *__restrict__ descs,
                                                        uint8_t *__restrict__ arena, uint8_t *__restrict__ exec,
                                                        const int64_t *__restrict__ exec_offs, const int vb,
                                                        DevError *err) {
    __shared__ MapTable s_mt;
    __shared__ EmitShared s;
    __shared__ int s_ok;
    const int64_t u = blockIdx.x;
    load_map_table(&s_mt, mt);
    __syncthreads();  // the table is read below by every thread
    const spreg_panel_desc sd = src_descs[u], d = descs[u];
    const int nk = s_mt.num_nkern;
    if (threadIdx.x == 0) {
        s_ok = (sd.values_off == d.values_off && sd.cols_off == d.cols_off && sd.counts_off == d.counts_off &&
                sd.num_values == d.num_values && sd.num_cols == d.num_cols) ? 1 : 0;
        if (!s_ok) raise_err(err, 8, u, 0);
    }
    __syncthreads();
    if (!s_ok) return;
    for (int64_t i = threadIdx.x; i < (int64_t)d.num_values * vb; i += CH)
        arena[d.values_off + i] = src[d.values_off + i];
    for (int64_t i = threadIdx.x; i < (int64_t)d.num_cols * 4; i += CH) arena[d.cols_off + i] = src[d.cols_off + i];
    uint8_t *xb = exec + exec_offs[u];
    emit_prologue(s, s_mt, unit_counts + u * nk, reinterpret_cast<int32_t *>(arena + d.counts_off), xb, vb);
    __syncthreads();
    const int32_t *cols = reinterpret_cast<const int32_t *>(src + d.cols_off);
    const uint8_t *vals = src + d.values_off;
    for (int id = 0; id < nk; ++id) {
        const int n = unit_counts[u * nk + id];
        const int pc = __popc(s_mt.id_to_pattern[id]);
        for (int r = threadIdx.x; r < n; r += CH) {
            reinterpret_cast<int32_t *>(xb + s.xcol[id])[r] = cols[s.start[id] + r];
            for (int q = 0; q < pc * vb; ++q)
                xb[s.xval[id] + (int64_t)r * pc * vb + q] = vals[((int64_t)s.vstart[id] + (int64_t)r * pc) * vb + q];
        }
    }
}

struct Scratch {
    int32_t *unit_counts = nullptr;
    UnitStats *stats = nullptr;
    unsigned *panel_maxabs = nullptr;
    unsigned long long *tile_nnz = nullptr;
    PackTotals *totals = nullptr;
    DevError *err = nullptr;
    int64_t *panel_work = nullptr;  // P work estimates
    int64_t *unit_xoff = nullptr;   // units execution-block offsets by unit
    unsigned long long *id_totals = nullptr;  // 256 entry counts by nanokernel id
    cudaStream_t s = nullptr;
    ~Scratch() {
        if (id_totals) cudaFreeAsync(id_totals, s);
        if (panel_work) cudaFreeAsync(panel_work, s);
        if (unit_xoff) cudaFreeAsync(unit_xoff, s);
        if (unit_counts) cudaFreeAsync(unit_counts, s);
        if (stats) cudaFreeAsync(stats, s);
        if (panel_maxabs) cudaFreeAsync(panel_maxabs, s);
        if (tile_nnz) cudaFreeAsync(tile_nnz, s);
        if (totals) cudaFreeAsync(totals, s);
        if (err) cudaFreeAsync(err, s);
    }
};

const char *dev_error_text(int code) {
    switch (code) {
    case 1: return "pattern code is not a nanokernel of this module";
    case 2: return "packer invariant num_nnz == padding + count_nonzero(panel) failed (mapping does not cover the pattern exactly once)";
    case 3: return "duplicate (row, column) entry in CSR input";
    case 4: return "column index out of range of the dense panel";
    case 5: return "imported descriptor addresses bytes outside the arena";
    case 6: return "imported nkern_counts do not add up to the unit's columns and values";
    case 7: return "imported column index outside the unit's K tile";
    case 8: return "imported descriptor differs from the layout of its counts";
    default: return "unknown device check";
    }
}

void release(spreg_packed *p) {
    if (!p) return;
    if (p->arena) cudaFree(p->arena);
    if (p->descs) cudaFree(p->descs);
    if (p->scales) cudaFree(p->scales);
    if (p->exec) cudaFree(p->exec);
    if (p->exec_offs) cudaFree(p->exec_offs);
    if (p->panel_order) cudaFree(p->panel_order);
    if (p->panel_rank) cudaFree(p->panel_rank);
    delete p;
}

// Shared tail of every pack: layout, totals, arena, scales, emit.
template <class EmitFn>
int finish_pack(const spreg_mapping *m, const Geom &g, int value_dtype, int64_t col_offset, int32_t m_tile,
                int32_t k_tile, Scratch &sc, const MapTable *mt_dev, EmitFn emit, spreg_packed **out,
                cudaStream_t stream) {
    const int nk = m->num_nkern;
    const int vb = dtype_bytes(value_dtype);
    spreg_packed *p = new spreg_packed();
    SPREG_CUDA(cudaGetDevice(&p->device));
    p->geom = g;
    for (int i = 0; i < 256; ++i) p->id_to_pattern[i] = (uint8_t)(i < nk ? m->id_to_pattern[i] : 0);
    const int64_t units = g.units;
    cudaError_t e = cudaMalloc(&p->descs, (size_t)(units > 0 ? units : 1) * sizeof(spreg_panel_desc));
    if (e == cudaSuccess) e = cudaMalloc(&p->exec_offs, (size_t)(units + 1) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&p->panel_order, (size_t)(g.P > 0 ? g.P : 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&p->panel_rank, (size_t)(g.P > 0 ? g.P : 1) * sizeof(int32_t));
    if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_NOMEM, "cudaMalloc(descs): %s", cudaGetErrorString(e)); }
    layout_kernel<<<1, 1024, 0, stream>>>(units, nk, vb, g.ppt, g.T, g.P, sc.stats, sc.tile_nnz, p->descs, sc.totals);
    std::vector<int64_t> work((size_t)g.P);
    if (g.P > 0) {
        panel_work_kernel<<<(unsigned)((g.P + 255) / 256), 256, 0, stream>>>(g.P, g.T, g.ppt, sc.stats, sc.panel_work);
        cudaMemcpyAsync(work.data(), sc.panel_work, (size_t)g.P * sizeof(int64_t), cudaMemcpyDeviceToHost, stream);
    }
    unsigned long long id_totals[256] = {};
    if (units > 0 && nk > 0) {
        id_totals_kernel<<<(unsigned)nk, 256, 0, stream>>>(sc.unit_counts, units, nk, sc.id_totals);
        cudaMemcpyAsync(id_totals, sc.id_totals, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream);
    }
    PackTotals tot;
    DevError derr;
    cudaMemcpyAsync(&tot, sc.totals, sizeof tot, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&derr, sc.err, sizeof derr, cudaMemcpyDeviceToHost, stream);
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_CUDA, "pack count/layout: %s", cudaGetErrorString(e)); }
    if (derr.code != 0) {
        release(p);
        SPREG_FAIL(SPREG_ERR_CHECK, "packer check failed at unit %d (value %d): %s", derr.unit, derr.value,
                   dev_error_text(derr.code));
    }
    for (int i = 0; i < 256; ++i) p->id_entries[i] = (int64_t)id_totals[i];
    // Panels by descending work (ties by index): the tile executor gives consecutive panels of this
    // order to the warps of one job, so a job's warps finish their K tiles at about the same time.
    {
        std::vector<int32_t> order((size_t)g.P), rank((size_t)g.P);
        for (int64_t i = 0; i < g.P; ++i) order[(size_t)i] = (int32_t)i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int32_t x, int32_t y) { return work[(size_t)x] > work[(size_t)y]; });
        for (int64_t i = 0; i < g.P; ++i) rank[(size_t)order[(size_t)i]] = (int32_t)i;
        p->work_desc.resize((size_t)g.P);
        for (int64_t i = 0; i < g.P; ++i) p->work_desc[(size_t)i] = work[(size_t)order[(size_t)i]];
        p->order_host = order;
        if (g.P > 0) {
            e = cudaMemcpyAsync(p->panel_order, order.data(), (size_t)g.P * sizeof(int32_t), cudaMemcpyHostToDevice,
                                stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(p->panel_rank, rank.data(), (size_t)g.P * sizeof(int32_t), cudaMemcpyHostToDevice,
                                    stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // the host vectors end with this scope
            if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_CUDA, "panel order: %s", cudaGetErrorString(e)); }
        }
    }
    exec_slots_kernel<<<1, 1024, 0, stream>>>(units, g.P, g.T, g.ppt, p->panel_order, sc.stats, p->exec_offs,
                                              sc.unit_xoff);
    const int64_t arena_bytes = tot.arena_bytes;
    e = cudaMalloc(&p->arena, (size_t)(arena_bytes > 0 ? arena_bytes : 64));
    if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_NOMEM, "cudaMalloc(arena %lld B): %s", (long long)arena_bytes, cudaGetErrorString(e)); }
    cudaMemsetAsync(p->arena, 0, (size_t)(arena_bytes > 0 ? arena_bytes : 64), stream);
    p->exec_bytes = tot.exec_bytes;
    p->max_exec_bytes = tot.max_exec_bytes;
    e = cudaMalloc(&p->exec, (size_t)(tot.exec_bytes > 0 ? tot.exec_bytes : 64));
    if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_NOMEM, "cudaMalloc(exec %lld B): %s", (long long)tot.exec_bytes, cudaGetErrorString(e)); }
    cudaMemsetAsync(p->exec, 0, (size_t)(tot.exec_bytes > 0 ? tot.exec_bytes : 64), stream);
    if (value_dtype == SPREG_F16) {
        e = cudaMalloc(&p->scales, (size_t)(g.P > 0 ? g.P : 1) * sizeof(float));
        if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_NOMEM, "cudaMalloc(scales): %s", cudaGetErrorString(e)); }
        if (g.P > 0) scales_kernel<<<(unsigned)((g.P + 255) / 256), 256, 0, stream>>>(g.P, sc.panel_maxabs, p->scales);
    }
    if (units > 0) emit(p);
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_CUDA, "pack emit: %s", cudaGetErrorString(e)); }

    spreg_packed_info &in = p->info;
    in.rows = g.M;
    in.cols = g.K;
    in.num_panels = g.P;
    in.num_units = units;
    in.mr = m->mr;
    in.num_nkern = nk;
    in.m_tile = m_tile;
    in.k_tile = k_tile;
    in.num_k_tiles = (int32_t)g.T;
    in.value_dtype = value_dtype;
    in.col_offset = col_offset;
    in.nnz = tot.nnz;
    in.num_values = tot.num_values;
    in.num_col_indices = tot.num_cols;
    in.padding = tot.padding;
    in.arena_bytes = arena_bytes;
    in.required_storage = tot.required_storage;
    in.algorithmic_bytes = tot.num_values * vb + tot.num_cols * 4 + (int64_t)units * nk * 4 +
                           units * (int64_t)sizeof(spreg_panel_desc) + (value_dtype == SPREG_F16 ? g.P * 4 : 0);
    in.empty_units = tot.empty_units;
    *out = p;
    return SPREG_OK;
}

int alloc_scratch(Scratch &sc, const Geom &g, int nk, int64_t tiles, cudaStream_t stream) {
    sc.s = stream;
    const int64_t units = g.units > 0 ? g.units : 1;
    SPREG_CUDA(cudaMallocAsync(&sc.unit_counts, (size_t)(units * (nk > 0 ? nk : 1)) * sizeof(int32_t), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.stats, (size_t)units * sizeof(UnitStats), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.panel_maxabs, (size_t)(g.P > 0 ? g.P : 1) * sizeof(unsigned), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.tile_nnz, (size_t)(tiles > 0 ? tiles : 1) * sizeof(unsigned long long), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.totals, sizeof(PackTotals), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.err, sizeof(DevError), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.panel_work, (size_t)(g.P > 0 ? g.P : 1) * sizeof(int64_t), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.unit_xoff, (size_t)units * sizeof(int64_t), stream));
    SPREG_CUDA(cudaMallocAsync(&sc.id_totals, 256 * sizeof(unsigned long long), stream));
    SPREG_CUDA(cudaMemsetAsync(sc.id_totals, 0, 256 * sizeof(unsigned long long), stream));
    SPREG_CUDA(cudaMemsetAsync(sc.panel_maxabs, 0, (size_t)(g.P > 0 ? g.P : 1) * sizeof(unsigned), stream));
    SPREG_CUDA(cudaMemsetAsync(sc.tile_nnz, 0, (size_t)(tiles > 0 ? tiles : 1) * sizeof(unsigned long long), stream));
    SPREG_CUDA(cudaMemsetAsync(sc.err, 0, sizeof(DevError), stream));
    SPREG_CUDA(cudaMemsetAsync(sc.totals, 0, sizeof(PackTotals), stream));
    return SPREG_OK;
}

int make_geom(const spreg_mapping *m, int64_t rows, int64_t cols, const spreg_pack_opts *o, Geom *g) {
    const int mr = m->mr;
    SPREG_CHECK_ARG(rows >= 0 && cols >= 0, "rows and cols must be non-negative");
    g->M = rows;
    g->K = cols;
    g->P = (rows + mr - 1) / mr;
    int32_t mt = o ? o->m_tile : 0, kt = o ? o->k_tile : 0;
    SPREG_CHECK_ARG(mt >= 0 && kt >= 0, "m_tile and k_tile must be non-negative");
    SPREG_CHECK_ARG(mt % mr == 0, "m_tile (%d) must be a multiple of M_r (%d) (count_nkerns.cpp:84-87)", mt, mr);
    g->ppt = mt > 0 ? mt / mr : (g->P > 0 ? g->P : 1);
    g->kt = kt > 0 ? kt : (cols > 0 ? cols : 1);
    g->T = cols > 0 ? (cols + g->kt - 1) / g->kt : 1;
    g->units = g->P * g->T;
    const int64_t co = o ? o->col_offset : 0;
    SPREG_CHECK_ARG(co >= 0 && cols + co <= INT32_MAX, "column indices (cols + col_offset) must fit int32");
    return SPREG_OK;
}

template <class Loader>
int pack_columns(const spreg_mapping *m, const Geom &g, const Loader &ld, const spreg_pack_opts *o,
                 spreg_packed **out, cudaStream_t stream) {
    int st = SPREG_OK;
    const MapTable *mt = mapping_device_table(m, &st);
    if (st != SPREG_OK) return st;
    const int value_dtype = o ? o->value_dtype : SPREG_F32;
    SPREG_CHECK_ARG(value_dtype >= SPREG_F32 && value_dtype <= SPREG_F16, "bad value dtype %d", value_dtype);
    const int64_t col_offset = o ? o->col_offset : 0;
    const int64_t tiles = (g.P > 0 ? (g.P + g.ppt - 1) / g.ppt : 0) * g.T;
    Scratch sc;
    st = alloc_scratch(sc, g, m->num_nkern, tiles, stream);
    if (st != SPREG_OK) return st;
    if (g.units > 0) {
        if (g.units > INT32_MAX) SPREG_FAIL(SPREG_ERR_UNSUPPORTED, "too many packed units");
        count_cols_kernel<Loader><<<(unsigned)g.units, CH, 0, stream>>>(g, ld, mt, sc.unit_counts, sc.stats,
                                                                          sc.panel_maxabs, sc.tile_nnz, sc.err,
                                                                          dtype_bytes(value_dtype));
        SPREG_CUDA(cudaGetLastError());
    }
    auto emit = [&](spreg_packed *p) {
        if (value_dtype == SPREG_F32)
            emit_cols_kernel<Loader, float><<<(unsigned)g.units, CH, 0, stream>>>(
                g, ld, mt, sc.unit_counts, p->descs, p->arena, nullptr, col_offset, p->exec, sc.unit_xoff);
        else if (value_dtype == SPREG_BF16)
            emit_cols_kernel<Loader, __nv_bfloat16><<<(unsigned)g.units, CH, 0, stream>>>(
                g, ld, mt, sc.unit_counts, p->descs, p->arena, nullptr, col_offset, p->exec, sc.unit_xoff);
        else
            emit_cols_kernel<Loader, __half><<<(unsigned)g.units, CH, 0, stream>>>(
                g, ld, mt, sc.unit_counts, p->descs, p->arena, p->scales, col_offset, p->exec, sc.unit_xoff);
    };
    return finish_pack(m, g, value_dtype, col_offset, o ? o->m_tile : 0, o ? o->k_tile : 0, sc, mt, emit, out, stream);
}

}  // namespace

int pack_dense_impl(const spreg_mapping *m, const float *a, int64_t rows, int64_t cols, int64_t lda,
                    const spreg_pack_opts *o, spreg_packed **out, cudaStream_t stream) {
    SPREG_CHECK_ARG(m && out, "null mapping or output");
    SPREG_CHECK_ARG(rows == 0 || cols == 0 || a, "null matrix");
    SPREG_CHECK_ARG(rows == 0 || lda >= cols, "lda (%lld) < cols (%lld)", (long long)lda, (long long)cols);
    Geom g;
    int st = make_geom(m, rows, cols, o, &g);
    if (st != SPREG_OK) return st;
    DenseLoader ld{a, lda, rows};
    return pack_columns(m, g, ld, o, out, stream);
}

int pack_csr_impl(const spreg_mapping *m, const spreg_csr *csr, const spreg_pack_opts *o, spreg_packed **out,
                  cudaStream_t stream) {
    SPREG_CHECK_ARG(m && csr && out, "null argument");
    SPREG_CHECK_ARG(csr->rows == 0 || csr->row_ptrs, "null row_ptrs");
    SPREG_CHECK_ARG(csr->nnz == 0 || (csr->col_inds && csr->values), "null col_inds / values");
    SPREG_CHECK_ARG(csr->nnz >= 0 && csr->nnz <= INT32_MAX, "nnz out of range");
    Geom g;
    int st = make_geom(m, csr->rows, csr->cols, o, &g);
    if (st != SPREG_OK) return st;
    CsrLoader ld{csr->row_ptrs, csr->col_inds, csr->values, csr->rows};
    return pack_columns(m, g, ld, o, out, stream);
}

// SOPTile path: panels staged on the host as (code, column) lists plus dense panels.
int pack_lists_impl(const spreg_mapping *m, int64_t rows, int64_t cols, int64_t num_panels,
                    const std::vector<int32_t> &codes, const std::vector<int32_t> &cols_in,
                    const std::vector<int64_t> &entry_off, const std::vector<float> &dense,
                    const std::vector<int64_t> &dense_off, const std::vector<int64_t> &panel_cols,
                    const std::vector<int64_t> &col_offsets, int value_dtype, spreg_packed **out,
                    cudaStream_t stream) {
    int st = SPREG_OK;
    const MapTable *mt = mapping_device_table(m, &st);
    if (st != SPREG_OK) return st;
    SPREG_CHECK_ARG(value_dtype >= SPREG_F32 && value_dtype <= SPREG_F16, "bad value dtype %d", value_dtype);
    Geom g;
    g.M = rows;
    g.K = cols;
    g.P = num_panels;
    g.ppt = num_panels > 0 ? num_panels : 1;
    g.T = 1;
    g.kt = cols > 0 ? cols : 1;
    g.units = num_panels;
    Scratch sc;
    st = alloc_scratch(sc, g, m->num_nkern, 1, stream);
    if (st != SPREG_OK) return st;

    // Upload staged lists.
    struct DevBuf {
        void *p = nullptr;
        cudaStream_t s;
        ~DevBuf() { if (p) cudaFreeAsync(p, s); }
    } b_codes{nullptr, stream}, b_cols{nullptr, stream}, b_eoff{nullptr, stream}, b_dense{nullptr, stream},
        b_doff{nullptr, stream}, b_pcols{nullptr, stream}, b_coff{nullptr, stream};
    auto up = [&](DevBuf &b, const void *src, size_t bytes) -> int {
        SPREG_CUDA(cudaMallocAsync(&b.p, bytes > 0 ? bytes : 16, stream));
        if (bytes) SPREG_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, stream));
        return SPREG_OK;
    };
    if ((st = up(b_codes, codes.data(), codes.size() * 4))) return st;
    if ((st = up(b_cols, cols_in.data(), cols_in.size() * 4))) return st;
    if ((st = up(b_eoff, entry_off.data(), entry_off.size() * 8))) return st;
    if ((st = up(b_dense, dense.data(), dense.size() * 4))) return st;
    if ((st = up(b_doff, dense_off.data(), dense_off.size() * 8))) return st;
    if ((st = up(b_pcols, panel_cols.data(), panel_cols.size() * 8))) return st;
    if ((st = up(b_coff, col_offsets.data(), col_offsets.size() * 8))) return st;
    ListSrc src{(const int32_t *)b_codes.p, (const int32_t *)b_cols.p, (const int64_t *)b_eoff.p,
                (const float *)b_dense.p, (const int64_t *)b_doff.p, (const int64_t *)b_pcols.p,
                (const int64_t *)b_coff.p};
    if (num_panels > 0) {
        count_list_kernel<<<(unsigned)num_panels, CH, 0, stream>>>(src, mt, sc.unit_counts, sc.stats,
                                                                    sc.panel_maxabs, sc.tile_nnz, sc.err,
                                                                    dtype_bytes(value_dtype));
        SPREG_CUDA(cudaGetLastError());
    }
    auto emit = [&](spreg_packed *p) {
        if (value_dtype == SPREG_F32)
            emit_list_kernel<float><<<(unsigned)num_panels, CH, 0, stream>>>(src, mt, sc.unit_counts, p->descs,
                                                                              p->arena, nullptr, p->exec, sc.unit_xoff);
        else if (value_dtype == SPREG_BF16)
            emit_list_kernel<__nv_bfloat16><<<(unsigned)num_panels, CH, 0, stream>>>(
                src, mt, sc.unit_counts, p->descs, p->arena, nullptr, p->exec, sc.unit_xoff);
        else
            emit_list_kernel<__half><<<(unsigned)num_panels, CH, 0, stream>>>(src, mt, sc.unit_counts, p->descs,
                                                                               p->arena, p->scales, p->exec, sc.unit_xoff);
    };
    st = finish_pack(m, g, value_dtype, 0, 0, 0, sc, mt, emit, out, stream);
    if (st == SPREG_OK && *out) (*out)->list_packed = true;
    return st;
}

int pack_from_arena_impl(const spreg_mapping *m, const spreg_arena_geom *ag, const void *arena_h,
                         int64_t arena_bytes, const spreg_panel_desc *descs_h, int64_t num_units,
                         const float *scales_h, int64_t num_scales, spreg_packed **out, cudaStream_t stream) {
    SPREG_CHECK_ARG(m && ag && out, "null argument");
    SPREG_CHECK_ARG(ag->value_dtype >= SPREG_F32 && ag->value_dtype <= SPREG_F16, "bad value dtype %d", ag->value_dtype);
    spreg_pack_opts o = {ag->m_tile, ag->k_tile, ag->col_offset, ag->value_dtype};
    Geom g;
    int st = make_geom(m, ag->rows, ag->cols, &o, &g);
    if (st != SPREG_OK) return st;
    SPREG_CHECK_ARG(num_units == g.units, "%lld descriptors for %lld units of this geometry", (long long)num_units,
                    (long long)g.units);
    SPREG_CHECK_ARG(arena_bytes >= 0 && (arena_bytes == 0 || arena_h) && (num_units == 0 || descs_h), "null arena");
    SPREG_CHECK_ARG(ag->value_dtype != SPREG_F16 || (scales_h && num_scales == g.P), "F16 arenas need %lld scales",
                    (long long)g.P);
    if (ag->value_dtype == SPREG_F16)
        for (int64_t i = 0; i < g.P; ++i)
            SPREG_CHECK_ARG(scales_h[i] > 0.0f && scales_h[i] < INFINITY, "scale %lld is not a finite positive value",
                            (long long)i);
    if (g.units > INT32_MAX) SPREG_FAIL(SPREG_ERR_UNSUPPORTED, "too many packed units");
    const MapTable *mt = mapping_device_table(m, &st);
    if (st != SPREG_OK) return st;
    const int vb = dtype_bytes(ag->value_dtype);
    const int64_t tiles = (g.P > 0 ? (g.P + g.ppt - 1) / g.ppt : 0) * g.T;
    Scratch sc;
    if ((st = alloc_scratch(sc, g, m->num_nkern, tiles, stream))) return st;
    struct DevBuf {
        void *p = nullptr;
        cudaStream_t s;
        ~DevBuf() { if (p) cudaFreeAsync(p, s); }
    } b_arena{nullptr, stream}, b_descs{nullptr, stream};
    SPREG_CUDA(cudaMallocAsync(&b_arena.p, (size_t)(arena_bytes > 0 ? arena_bytes : 16), stream));
    SPREG_CUDA(cudaMallocAsync(&b_descs.p, (size_t)(num_units > 0 ? num_units : 1) * sizeof(spreg_panel_desc), stream));
    if (arena_bytes) SPREG_CUDA(cudaMemcpyAsync(b_arena.p, arena_h, (size_t)arena_bytes, cudaMemcpyHostToDevice, stream));
    if (num_units)
        SPREG_CUDA(cudaMemcpyAsync(b_descs.p, descs_h, (size_t)num_units * sizeof(spreg_panel_desc),
                                   cudaMemcpyHostToDevice, stream));
    const uint8_t *src = static_cast<const uint8_t *>(b_arena.p);
    const spreg_panel_desc *sdesc = static_cast<const spreg_panel_desc *>(b_descs.p);
    if (g.units > 0) {
        arena_count_kernel<<<(unsigned)g.units, CH, 0, stream>>>(g, mt, src, arena_bytes, sdesc, vb, ag->col_offset,
                                                                 sc.unit_counts, sc.stats, sc.tile_nnz, sc.err);
        SPREG_CUDA(cudaGetLastError());
    }
    auto emit = [&](spreg_packed *p) {
        arena_emit_kernel<<<(unsigned)g.units, CH, 0, stream>>>(mt, src, sdesc, sc.unit_counts, p->descs, p->arena,
                                                                p->exec, sc.unit_xoff, vb, sc.err);
    };
    spreg_packed *p = nullptr;
    st = finish_pack(m, g, ag->value_dtype, ag->col_offset, ag->m_tile, ag->k_tile, sc, mt, emit, &p, stream);
    if (st != SPREG_OK) return st;
    DevError derr;
    cudaError_t e = cudaMemcpyAsync(&derr, sc.err, sizeof derr, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess && ag->value_dtype == SPREG_F16 && g.P > 0)
        e = cudaMemcpyAsync(p->scales, scales_h, (size_t)g.P * sizeof(float), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { release(p); SPREG_FAIL(SPREG_ERR_CUDA, "arena import: %s", cudaGetErrorString(e)); }
    if (derr.code != 0) {
        release(p);
        SPREG_FAIL(SPREG_ERR_CHECK, "arena import check failed at unit %d (value %d): %s", derr.unit, derr.value,
                   dev_error_text(derr.code));
    }
    if (p->info.arena_bytes != arena_bytes) {
        const long long want = (long long)p->info.arena_bytes;
        release(p);
        SPREG_FAIL(SPREG_ERR_CHECK, "arena holds %lld bytes, its descriptors lay out %lld", (long long)arena_bytes, want);
    }
    *out = p;
    return SPREG_OK;
}

int sort_encode_impl(const spreg_mapping *m, const int32_t *codes, int64_t n, int32_t *encoded, int32_t *order,
                     cudaStream_t stream) {
    SPREG_CHECK_ARG(m, "null mapping");
    SPREG_CHECK_ARG(n >= 0 && n <= INT32_MAX, "n out of range");
    SPREG_CHECK_ARG(n == 0 || (codes && encoded && order), "null array");
    if (n == 0) return SPREG_OK;
    int st = SPREG_OK;
    const MapTable *mt = mapping_device_table(m, &st);
    if (st != SPREG_OK) return st;
    DevError *err = nullptr;
    SPREG_CUDA(cudaMallocAsync(&err, sizeof(DevError), stream));
    cudaMemsetAsync(err, 0, sizeof(DevError), stream);
    sort_encode_kernel<<<1, CH, 0, stream>>>(mt, codes, n, encoded, order, err);
    DevError h;
    cudaMemcpyAsync(&h, err, sizeof h, cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(err, stream);
    SPREG_CUDA(cudaStreamSynchronize(stream));
    if (h.code) SPREG_FAIL(SPREG_ERR_CHECK, "sort_and_encode_patterns: entry %d has code %d: %s", h.unit, h.value,
                           dev_error_text(h.code));
    return SPREG_OK;
}

void packed_release(spreg_packed *p) { release(p); }

}  // namespace spreg
