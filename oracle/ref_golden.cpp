// ref_golden.cpp -- builds the reference's own host-side format code from the
// AccSpMM sources (include/mmio.hpp, include/format.hpp, include/utils.hpp,
// found through -I at build time, never copied) and dumps what it produces for
// one Matrix Market file.  TEST INFRASTRUCTURE ONLY: it is the pin for the
// oracle and for the product's builders, run here to make committed fixtures.
//
// usage: ref_golden <matrix.mtx> <out.bin>
// out.bin: a sequence of records {char name[16]; uint32 dtype; uint64 count;
// payload}, dtype 1 = uint32, 2 = uint64, 3 = float32, 4 = int32.
#include "mmio.hpp"
#include "utils.hpp"

#include <cstdio>
#include <vector>

static void put(FILE* f, const char* name, uint32_t dtype, uint64_t count,
                const void* data, size_t elem) {
    char n[16] = {0};
    std::snprintf(n, sizeof n, "%s", name);
    std::fwrite(n, 1, 16, f);
    std::fwrite(&dtype, 4, 1, f);
    std::fwrite(&count, 8, 1, f);
    if (count) std::fwrite(data, elem, count, f);
}

int main(int argc, char** argv) {
    if (argc < 3) return 4;
    COO<float> coo;
    int status = read_from_mtx<float>(argv[1], &coo);
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    put(f, "status", 4, 1, &status, 4);
    if (status != SUCCESS) { std::fclose(f); return 0; }
    uint32_t dims[3] = {coo.rows, coo.cols, coo.nnz};
    put(f, "dims", 1, 3, dims, 4);
    put(f, "coo_row", 1, coo.nnz, coo.row, 4);
    put(f, "coo_col", 1, coo.nnz, coo.col, 4);
    put(f, "coo_data", 3, coo.nnz, coo.data, 4);

    CSR<float> csr(&coo);
    put(f, "csr_row_ptr", 1, csr.row_ptr.size(), csr.row_ptr.data(), 4);
    put(f, "csr_col_idx", 1, csr.col_idx.size(), csr.col_idx.data(), 4);
    put(f, "csr_data", 3, csr.data.size(), csr.data.data(), 4);

    METCFBit<float> m;
    m.convertFromCSR(csr);
    put(f, "m_rwo", 1, m.rowWindowOffset.size(), m.rowWindowOffset.data(), 4);
    put(f, "m_tc_offset", 1, m.tcOffset.size(), m.tcOffset.data(), 4);
    put(f, "m_bits", 2, m.tcLocalBit.size(), m.tcLocalBit.data(), 8);
    put(f, "m_a2b", 1, m.sparseA2B.size(), m.sparseA2B.data(), 4);
    put(f, "m_data", 3, m.data.size(), m.data.data(), 4);

    if (m.rowWindowOffset.size() > 1) {
        int adaptive = balanceStrategy(m, m.tcOffset.size() - 1,
                                       m.rowWindowOffset.size() - 1) ? 1 : 0;
        put(f, "balance", 4, 1, &adaptive, 4);
    }
    if (m.tcOffset.size() > 1) {
        // the reference's driver call, src/mma_tf32.cu:222
        AdpBME<float> a;
        a.CSR2AdpBME(csr, 3, 1, 2);
        put(f, "a_group_offset", 1, a.groupOffset.size(), a.groupOffset.data(), 4);
        put(f, "a_tc_offset", 1, a.tcOffset.size(), a.tcOffset.data(), 4);
        put(f, "a_row_indices", 1, a.rowIndices.size(), a.rowIndices.data(), 4);
        put(f, "a_bits", 2, a.tcLocalBit.size(), a.tcLocalBit.data(), 8);
        put(f, "a_a2b", 1, a.sparseA2B.size(), a.sparseA2B.data(), 4);
        put(f, "a_data", 3, a.data.size(), a.data.data(), 4);
        // a second parameter set, to pin the grouping rule beyond the default
        AdpBME<float> b;
        b.CSR2AdpBME(csr, 2, 3, 5, 4);
        put(f, "b_group_offset", 1, b.groupOffset.size(), b.groupOffset.data(), 4);
    }
    std::fclose(f);
    return 0;
}
