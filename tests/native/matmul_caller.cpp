// Native caller of libspreg's C ABI, in the order the reference's C++ testbed drives
// sop::MatMulSpecialized (cpp_testbed/src/spmm/nano/SpMM_SOP.h:107-178): a mapping, the matmul built
// from a host CSR matrix and a TileConfig, allocate_executor(n), then operator()(C, B) with host
// buffers, synchronous and enqueued.  Only include/spreg.h and the shared library are used.
//
//   matmul_caller cpu   argument and error paths (no GPU call)
//   matmul_caller gpu   C = A.B for a 300 x 520 CSR A at 90 % sparsity and B 520 x 96, checked
//                       against a double-precision CSR product computed here (rel err <= 1e-5)
// Prints "ok ..." and exits 0 when every check passes.
#include "spreg.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

namespace {

int failed(const char *what) {
    std::fprintf(stderr, "FAIL %s: %s\n", what, spreg_last_error());
    return 1;
}

// Identity mapping of M_r-bit patterns: pattern p -> [p], pattern 0 -> no nanokernel.
spreg_mapping *identity_mapping(int mr) {
    std::vector<int32_t> offs((1 << mr) + 1), codes;
    for (int p = 0; p < (1 << mr); ++p) {
        offs[p] = (int32_t)codes.size();
        if (p) codes.push_back(p);
    }
    offs[1 << mr] = (int32_t)codes.size();
    spreg_mapping *m = nullptr;
    return spreg_mapping_create(mr, offs.data(), codes.data(), nullptr, 0, &m) == SPREG_OK ? m : nullptr;
}

int cpu_checks() {
    spreg_mapping *m = identity_mapping(4);
    if (!m) return failed("identity mapping");
    if (spreg_mapping_num_nkern(m) != 15) return failed("15 nanokernels");
    std::vector<int32_t> offs(9, 0);
    spreg_mapping *bad = nullptr;
    if (spreg_mapping_create(3, offs.data(), offs.data(), nullptr, 0, &bad) != SPREG_ERR_INVALID_ARG || bad ||
        std::strlen(spreg_last_error()) == 0)
        return failed("M_r = 3 refused with a message");
    spreg_mapping_destroy(m);
    std::printf("ok cpu\n");
    return 0;
}

int gpu_checks() {
    const int M = 300, K = 520, N = 96;
    std::mt19937 gen(7);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    std::normal_distribution<float> nrm(0.0f, 1.0f);
    std::vector<int32_t> rp(M + 1, 0), ci;
    std::vector<float> vals;
    for (int r = 0; r < M; ++r) {
        for (int c = 0; c < K; ++c)
            if (u01(gen) < 0.1f) {
                ci.push_back(c);
                vals.push_back(nrm(gen));
            }
        rp[r + 1] = (int32_t)ci.size();
    }
    std::vector<float> B((size_t)K * N), C((size_t)M * N, -1.0f), C2((size_t)M * N, -1.0f);
    for (float &b : B) b = nrm(gen);
    std::vector<double> want((size_t)M * N, 0.0);
    for (int r = 0; r < M; ++r)
        for (int e = rp[r]; e < rp[r + 1]; ++e)
            for (int j = 0; j < N; ++j) want[(size_t)r * N + j] += (double)vals[e] * (double)B[(size_t)ci[e] * N + j];

    spreg_mapping *m = identity_mapping(4);
    if (!m) return failed("identity mapping");
    spreg_tile_config cfg = {};
    cfg.m_tile = 16;   // SOPConfig defaults (SpMM_SOP.h:33-54): m_tile 16, k_tile 256, n_tile 64
    cfg.k_tile = 256;
    cfg.n_tile = 64;
    cfg.value_dtype = SPREG_F32;
    cfg.beta_10x = 10;
    spreg_matmul *mm = nullptr;
    if (spreg_matmul_create(M, K, N, vals.data(), rp.data(), ci.data(), &cfg, m, &mm) != SPREG_OK)
        return failed("matmul create");
    if (spreg_matmul_allocate_executor(mm, N) != SPREG_OK) return failed("allocate_executor");
    if (spreg_matmul_required_storage(mm) <= 0) return failed("require_storage");
    if (spreg_matmul_run(mm, C.data(), B.data()) != SPREG_OK) return failed("operator()(C, B)");
    if (spreg_matmul_run_async(mm, C2.data(), B.data()) != SPREG_OK || spreg_matmul_sync(mm) != SPREG_OK)
        return failed("enqueued operator()(C, B)");
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < want.size(); ++i) {
        num += (C[i] - want[i]) * (C[i] - want[i]);
        den += want[i] * want[i];
        if (std::memcmp(&C[i], &C2[i], sizeof(float)) != 0) return failed("enqueued call differs");
    }
    const double rel = std::sqrt(num / den);
    if (!(rel <= 1e-5)) {
        std::fprintf(stderr, "FAIL rel err %.3e\n", rel);
        return 1;
    }
    int32_t status = 0;
    if (spreg_device_status(&status, 0) != SPREG_OK || status != 0) return failed("device status");
    spreg_matmul_destroy(mm);
    spreg_mapping_destroy(m);
    std::printf("ok gpu rel_err %.3e nnz %zu\n", rel, vals.size());
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc > 1 && std::strcmp(argv[1], "gpu") == 0) return gpu_checks();
    return cpu_checks();
}
