// mma_main.cpp -- the `mma <matrix.mtx> <feature_dim>` command of
// src/mma_tf32.cu:185-243, rebuilt on the C ABI.
//
// Same argv, exit codes (4 = ERROR_ARGS, 3 = ERROR_READ_MTX, 0 = success) and
// the same line appended to ./result.csv: "<file name>,<K>,<avg ms>,<GFLOP/s>"
// with GFLOP/s = 2 nnz K / t (src/mma_tf32.cu:231-239).  The flow follows the
// reference: load, CSR, METCF, balanceStrategy, then the adaptive (AdpBME with
// parameters 3, 1, 2) or the plain kernel, 10 warm-up + 10 timed launches with
// B = 1.0 (src/mma_tf32.cu:44).  METCF and AdpBME are built on the GPU.
// Extra options, after the two positional arguments:
//   --precision tf32|3xtf32   arithmetic (default tf32)
//   --host-build              build METCF / AdpBME on the host instead
//   --metcf-cache             load METCF from <matrix.mtx>.metcf when that
//                             file is newer than the .mtx; otherwise build it
//                             and write the file for the next run
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "accspmm.h"

static std::string base_name(const std::string& s) {
    size_t p = s.rfind('/');
    return p == std::string::npos ? s : s.substr(p + 1);
}

// modification time, or -1 if the file does not exist
static long long mtime_of(const std::string& path) {
    struct stat sb;
    if (stat(path.c_str(), &sb) != 0) return -1;
    return (long long)sb.st_mtime;
}

static int fail(const char* what, int st) {
    std::fprintf(stderr, "mma: %s failed (status %d): %s\n", what, st, accspmm_last_error());
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::printf("Usage: ./mma <matrix.mtx> <feature_dim>\n");
        return ACCSPMM_ERROR_ARGS;
    }
    const char* filename = argv[1];
    const int feature_dim = std::atoi(argv[2]);
    int precision = ACCSPMM_PREC_TF32;
    bool host_build = false;
    bool metcf_cache = false;
    for (int i = 3; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--precision") && i + 1 < argc) {
            precision = !std::strcmp(argv[++i], "3xtf32") ? ACCSPMM_PREC_3XTF32 : ACCSPMM_PREC_TF32;
        } else if (!std::strcmp(argv[i], "--host-build")) {
            host_build = true;
        } else if (!std::strcmp(argv[i], "--metcf-cache")) {
            metcf_cache = true;
        }
    }
    if (feature_dim <= 0 || feature_dim % 4) {
        std::fprintf(stderr, "mma: feature_dim must be a positive multiple of 4\n");
        return ACCSPMM_ERROR_ARGS;
    }
    const uint32_t K = uint32_t(feature_dim);
    const std::string mtx_name = base_name(filename);

    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    const std::string cache_path = std::string(filename) + ".metcf";
    accspmm_metcf_t m;
    int st = 1;
    if (metcf_cache && mtime_of(cache_path) >= mtime_of(filename) && mtime_of(filename) >= 0) {
        st = accspmm_metcf_load(cache_path.c_str(), ACCSPMM_DEVICE, &m, s);
        if (st) std::fprintf(stderr, "mma: ignoring %s: %s\n", cache_path.c_str(), accspmm_last_error());
        else std::cout << "loaded " << cache_path << std::endl;
    }
    if (st) {
        accspmm_coo_t coo;
        st = accspmm_read_mtx(filename, &coo);
        if (st != ACCSPMM_SUCCESS) {
            std::fprintf(stderr, "mma: %s\n", accspmm_last_error());
            return ACCSPMM_ERROR_READ_MTX;
        }
        std::cout << "m_tmp: " << coo.rows << ", n_tmp: " << coo.cols << ", nnz_tmp: " << coo.nnz << std::endl;

        accspmm_csr_t csr;
        if ((st = accspmm_csr_from_coo(&coo, &csr, s))) return fail("csr_from_coo", st);
        accspmm_coo_destroy(&coo);

        if (host_build) {
            accspmm_metcf_t hm;
            if ((st = accspmm_metcf_from_csr(&csr, &hm, s))) return fail("metcf_from_csr", st);
            if ((st = accspmm_metcf_copy(&hm, ACCSPMM_DEVICE, &m, s))) return fail("metcf_copy", st);
            accspmm_metcf_destroy(&hm);
        } else {
            accspmm_csr_t dcsr;
            if ((st = accspmm_csr_copy(&csr, ACCSPMM_DEVICE, &dcsr, s))) return fail("csr_copy", st);
            if ((st = accspmm_metcf_from_csr(&dcsr, &m, s))) return fail("metcf_from_csr", st);
            accspmm_csr_destroy(&dcsr);
        }
        accspmm_csr_destroy(&csr);
        if (metcf_cache && (st = accspmm_metcf_save(&m, cache_path.c_str(), s)))
            std::fprintf(stderr, "mma: could not write %s: %s\n", cache_path.c_str(), accspmm_last_error());
    }
    // nnz after symmetric expansion: the METCF holds exactly the CSR's values
    const uint32_t num_edges = m.nnz;

    int adaptive = 0;
    if ((st = accspmm_balance_strategy(&m, &adaptive, s))) return fail("balance_strategy", st);

    accspmm_adpbme_t adp;
    std::memset(&adp, 0, sizeof adp);
    uint32_t c_rows = m.num_windows * 8;
    if (adaptive) {
        if ((st = accspmm_adpbme_from_metcf(&m, 3, 1, 2, 16, &adp, s))) return fail("adpbme", st);
        if ((st = accspmm_adaptive_c_rows(&adp, &c_rows, s))) return fail("adaptive_c_rows", st);
    }
    std::vector<float> hb(size_t(m.cols) * K, 1.0f);
    float *dB = nullptr, *dC = nullptr;
    if (cudaMalloc(&dB, hb.size() * 4 + 16) != cudaSuccess ||
        cudaMalloc(&dC, size_t(c_rows) * K * 4 + 16) != cudaSuccess) {
        std::fprintf(stderr, "mma: device allocation failed\n");
        return 1;
    }
    cudaMemcpyAsync(dB, hb.data(), hb.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(dC, 0, size_t(c_rows) * K * 4, s);
    std::cout << (adaptive ? "doing AdpBalance pipelining ..." : "doing pipelining mma ...") << std::endl;
    float elapsed_time = 0.f;
    st = accspmm_time_spmm(adaptive ? nullptr : &m, adaptive ? &adp : nullptr, dB, dC, c_rows, K,
                           precision, 10, 10, &elapsed_time, s);
    if (st) return fail("spmm", st);
    std::vector<float> hc(size_t(c_rows) * K);
    cudaMemcpyAsync(hc.data(), dC, hc.size() * 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);

    float spmm_throughput = (float(num_edges) * float(feature_dim) * 2.0f * 1000.f) /
                            (elapsed_time * 1000.f * 1000.f * 1000.f);
    std::ofstream out("result.csv", std::ios::app);
    if (!out) std::cerr << "Error Opening result.csv" << std::endl;
    out << mtx_name << "," << feature_dim << "," << elapsed_time << "," << spmm_throughput << "\n";
    out.close();

    cudaFree(dB);
    cudaFree(dC);
    accspmm_adpbme_destroy(&adp);
    accspmm_metcf_destroy(&m);
    cudaStreamDestroy(s);
    return 0;
}
