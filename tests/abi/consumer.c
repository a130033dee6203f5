/* consumer.c -- a C99 program that uses libaccspmm.so through include/accspmm.h
 * only, as a C caller of the reference's host path would: Matrix Market file
 * -> COO -> CSR -> METCF -> balance decision -> AdpBME, all on the host (no
 * GPU needed).  It prints the sizes and the first tile's column list, so a
 * test can compare them with the reference's known answers.  Test
 * infrastructure: compiled and run by tests/test_abi_c.py.
 *
 *   usage: consumer <matrix.mtx>
 *   exit:  0 on success, the library's status code otherwise */
#include <stdio.h>

#include "accspmm.h"

static int fail(const char* what, int st) {
    fprintf(stderr, "%s: status %d: %s\n", what, st, accspmm_last_error());
    return st;
}

int main(int argc, char** argv) {
    accspmm_coo_t coo;
    accspmm_csr_t csr;
    accspmm_metcf_t metcf;
    accspmm_adpbme_t adp;
    int adaptive = -1, st;
    uint32_t i;
    if (argc < 2) return ACCSPMM_ERROR_ARGS;
    st = accspmm_read_mtx(argv[1], &coo);
    if (st != ACCSPMM_SUCCESS) return fail("read", st);
    st = accspmm_csr_from_coo(&coo, &csr, NULL);
    if (st != ACCSPMM_SUCCESS) return fail("csr", st);
    st = accspmm_metcf_from_csr(&csr, &metcf, NULL);
    if (st != ACCSPMM_SUCCESS) return fail("metcf", st);
    st = accspmm_balance_strategy(&metcf, &adaptive, NULL);
    if (st != ACCSPMM_SUCCESS) return fail("balance", st);
    st = accspmm_adpbme_from_metcf(&metcf, 3, 1, 2, 16, &adp, NULL);
    if (st != ACCSPMM_SUCCESS) return fail("adpbme", st);
    printf("rows %u cols %u nnz %u windows %u tiles %u groups %u adaptive %d\n", metcf.rows,
           metcf.cols, metcf.nnz, metcf.num_windows, metcf.num_tiles, adp.num_groups, adaptive);
    printf("a2b");
    for (i = 0; i < 8 * metcf.num_tiles; ++i) {
        if (metcf.sparse_a2b[i] == 0xFFFFFFFFu) printf(" -");
        else printf(" %u", metcf.sparse_a2b[i]);
    }
    printf("\ndata");
    for (i = 0; i < metcf.nnz; ++i) printf(" %g", (double)metcf.data[i]);
    printf("\n");
    accspmm_adpbme_destroy(&adp);
    accspmm_metcf_destroy(&metcf);
    accspmm_csr_destroy(&csr);
    accspmm_coo_destroy(&coo);
    return 0;
}
