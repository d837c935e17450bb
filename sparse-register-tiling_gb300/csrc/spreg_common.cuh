// spreg_common.cuh -- types shared by the packer, the executor and the C ABI of libspreg.so.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/spreg.h"

namespace spreg {

// ------------------------------------------------------------------ error plumbing
void set_error(const std::string &msg);
void clear_error();

struct Status {
    int code = SPREG_OK;
    static Status ok() { return Status(); }
};

#define SPREG_FAIL(code, ...)                                                    \
    do {                                                                         \
        char _buf[512];                                                          \
        snprintf(_buf, sizeof _buf, __VA_ARGS__);                                \
        ::spreg::set_error(_buf);                                                \
        return (code);                                                           \
    } while (0)

#define SPREG_CUDA(call)                                                         \
    do {                                                                         \
        cudaError_t _e = (call);                                                 \
        if (_e != cudaSuccess) {                                                 \
            SPREG_FAIL(_e == cudaErrorMemoryAllocation ? SPREG_ERR_NOMEM : SPREG_ERR_CUDA, \
                       "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
        }                                                                        \
    } while (0)

#define SPREG_CHECK_ARG(cond, ...)                                               \
    do {                                                                         \
        if (!(cond)) SPREG_FAIL(SPREG_ERR_INVALID_ARG, __VA_ARGS__);             \
    } while (0)

// ------------------------------------------------------------------ mapping table
constexpr uint16_t kCodeInvalid = 0xFFFE;
constexpr uint16_t kCodeZero = SPREG_ZERO_PATTERN_ID;
constexpr int kMaxCodesPerPattern = SPREG_MAX_MR;

// Device copy of one nanokernel set + pattern mapping.  Patterns and codes are < 256.
struct MapTable {
    int32_t mr;
    int32_t num_nkern;
    uint16_t code_to_id[256];        // id, kCodeZero for 0, kCodeInvalid if not a nanokernel
    uint8_t id_to_pattern[256];      // nanokernel pattern of an id
    uint8_t map_n[256];              // number of (nonzero) codes a pattern maps to
    uint8_t map_codes[256][kMaxCodesPerPattern];
};

// ------------------------------------------------------------------ packed geometry
// Units (panel x K tile) are ordered row tile, K tile, panel (count_nkerns.cpp:78-125).
struct Geom {
    int64_t M, K;      // rows, columns of A
    int64_t P;         // row panels
    int64_t ppt;       // panels per row tile
    int64_t T;         // K tiles
    int64_t kt;        // columns per K tile
    int64_t units;     // P * T
};

__host__ __device__ inline int64_t unit_index(int64_t gp, int64_t tj, int64_t ppt, int64_t T, int64_t P) {
    const int64_t ti = gp / ppt;
    const int64_t p_lo = ti * ppt;
    const int64_t n_in = (p_lo + ppt < P) ? ppt : (P - p_lo);
    return p_lo * T + tj * n_in + (gp - p_lo);
}

// Execution blocks lie in slot order: K tile major, then panels by descending work (panel_rank),
// so the blocks of consecutive panels in that order at one K tile are adjacent in memory.
__host__ __device__ inline int64_t exec_slot(int64_t gp, int64_t tj, int64_t P, const int32_t *panel_rank) {
    return tj * P + panel_rank[gp];
}

// Inverse of unit_index: unit -> (global panel, K tile).
__host__ __device__ inline void unit_coords(int64_t u, int64_t ppt, int64_t T, int64_t P, int64_t *gp, int64_t *tj) {
    const int64_t per_tile = ppt * T;
    const int64_t ti = u / per_tile;
    const int64_t p_lo = ti * ppt;
    const int64_t n_in = (p_lo + ppt < P) ? ppt : (P - p_lo);
    const int64_t rem = u - p_lo * T;
    *tj = rem / n_in;
    *gp = p_lo + (rem - *tj * n_in);
}

__host__ __device__ inline int64_t align64(int64_t x) { return (x + 63) & ~int64_t(63); }
inline int dtype_bytes(int dt) { return dt == SPREG_F32 ? 4 : 2; }

// ------------------------------------------------------------------ dtype helpers
template <class T> struct DT;
template <> struct DT<float> {
    static constexpr int id = SPREG_F32;
    __device__ static float to_f32(float v) { return v; }
    __device__ static float from_f32(float v) { return v; }
};
template <> struct DT<__nv_bfloat16> {
    static constexpr int id = SPREG_BF16;
    __device__ static float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static __nv_bfloat16 from_f32(float v) { return __float2bfloat16_rn(v); }
};
template <> struct DT<__half> {
    static constexpr int id = SPREG_F16;
    __device__ static float to_f32(__half v) { return __half2float(v); }
    __device__ static __half from_f32(float v) { return __float2half_rn(v); }
};

// Per-unit statistics written by the count pass.
struct UnitStats {
    int32_t num_cols;    // entries U
    int32_t num_values;  // values V (nnz + padding)
    int32_t padding;     // emitted zeros
    int32_t nnz;         // nonzeros of the unit's dense panel slice
    int32_t exec_bytes;  // bytes of the unit's execution block
    int32_t num_groups;  // ids with a nonzero count
};

// Execution layout: per unit a 16-byte-aligned block read by the executor in one bulk copy:
//   [ExecHeader][ExecGroup x num_groups][per group: cols (pad to 4 entries) | values (pad to 4 entries, 16 B)]
// Groups are the ids with a nonzero count, in id order; every group's cols and values start on a
// 16-byte boundary, so the executor fetches the indices and values of 4 entries with vector loads.
struct ExecHeader {
    uint32_t num_groups, block_bytes, pad0, pad1;
};
struct ExecGroup {
    uint32_t pattern, count, cols_off, vals_off;  // offsets in bytes from the block start
};
constexpr int kExecPad = 4;  // entries per group are padded to a multiple of this
__host__ __device__ inline int64_t pad_entries(int64_t n) { return (n + kExecPad - 1) / kExecPad * kExecPad; }
// Bytes of a group's cols and values sections in the execution block.
__host__ __device__ inline int64_t exec_cols_bytes(int64_t n) { return pad_entries(n) * 4; }
__host__ __device__ inline int64_t exec_vals_bytes(int64_t n, int pc, int vb) {
    return (pad_entries(n) * pc * vb + 15) / 16 * 16;
}

// Totals written by the layout pass (one struct, copied to the host once).
struct PackTotals {
    long long arena_bytes;
    long long num_values;
    long long num_cols;
    long long padding;
    long long nnz;
    long long required_storage;
    long long empty_units;
    long long exec_bytes;      // execution layout bytes
    long long max_exec_bytes;  // largest execution block of one unit
};

// Device-side check words: first failing unit / code.
struct DevError {
    int32_t code;   // 0 ok; 1 bad code; 2 invariant; 3 duplicate csr entry; 4 column out of range
    int32_t unit;
    int32_t value;
    int32_t pad;
};

}  // namespace spreg

// Opaque handle definitions (C ABI types).
struct spreg_mapping {
    int32_t mr = 0;
    int32_t num_nkern = 0;
    int32_t id_to_pattern[256] = {};
    int32_t code_to_id[256] = {};   // -1 invalid, SPREG_ZERO_PATTERN_ID for 0
    spreg::MapTable host;           // table uploaded to devices
    void *dev[64] = {};             // per-device copy of `host`
};

struct spreg_packed {
    int device = -1;
    spreg_packed_info info = {};
    spreg::Geom geom = {};
    uint8_t *arena = nullptr;
    spreg_panel_desc *descs = nullptr;
    float *scales = nullptr;
    uint8_t id_to_pattern[256] = {};
    uint8_t *exec = nullptr;        // execution layout (derived from the arena by the packer)
    int64_t *exec_offs = nullptr;   // units + 1 block offsets, in slot order (exec_slot)
    int32_t *panel_order = nullptr; // P panels by descending work: slot t * P + i holds unit (panel_order[i], t)
    int32_t *panel_rank = nullptr;  // inverse of panel_order
    int64_t id_entries[256] = {};   // packed entries (columns) of each nanokernel id, all units
    int64_t exec_bytes = 0;
    int64_t max_exec_bytes = 0;
    bool list_packed = false;       // packed panel by panel (per-panel column offsets, no K tiles)
    std::vector<int64_t> work_desc; // the panels' work estimates in panel_order (descending), host copy
    std::vector<int32_t> order_host; // panel_order, host copy
};
