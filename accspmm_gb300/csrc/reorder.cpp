// reorder.cpp -- locality reordering of a square sparse matrix before METCF.
//
// METCF packs each 8-row window's distinct columns into 8-column tiles, so
// the number of tiles -- and the B rows the SpMM gathers -- falls when the
// rows of a window share columns, and the gathers hit L2 more often when
// neighbouring windows touch nearby B rows.  Both improve when the matrix is
// renumbered so that connected vertices get close numbers.  The reference
// ships no such pass; its benchmark input (a "my_reorder" matrix) was
// reordered offline.  This file provides reverse Cuthill-McKee (Cuthill &
// McKee 1969, reversed as proposed by George 1971, with the pseudo-peripheral
// start vertex of Gibbs, Poole & Stockmeyer 1976) on the symmetrised pattern
// A + A^T, and the symmetric permutation P A P^T of a CSR matrix.
//
// Convention: perm[new] = old.  With A' = P A P^T (A'[i', j'] = A[perm[i'],
// perm[j']]), A B = P^T (A' (P B)): gather B's rows by perm, multiply, and
// scatter the product's rows back by perm (accspmm_dense_permute_rows).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "accspmm.h"
#include "common.hpp"
#include "host_formats.hpp"

namespace accspmm {

namespace {

// Symmetrised adjacency (no self loops, no duplicates) in CSR form.
struct Graph {
    std::vector<uint64_t> ptr;
    std::vector<uint32_t> adj;
    uint32_t n = 0;
    uint32_t degree(uint32_t v) const { return uint32_t(ptr[v + 1] - ptr[v]); }
};

Graph symmetrise(const accspmm_csr_t* a) {
    Graph g;
    const uint32_t n = a->rows;
    g.n = n;
    std::vector<uint64_t> cnt(size_t(n) + 1, 0);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t p = a->row_ptr[i]; p < a->row_ptr[i + 1]; ++p) {
            const uint32_t j = a->col_idx[p];
            if (j == i) continue;
            ++cnt[i + 1];
            ++cnt[size_t(j) + 1];
        }
    for (size_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<uint32_t> raw(cnt[n]);
    std::vector<uint64_t> fill(cnt.begin(), cnt.end() - 1);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t p = a->row_ptr[i]; p < a->row_ptr[i + 1]; ++p) {
            const uint32_t j = a->col_idx[p];
            if (j == i) continue;
            raw[fill[i]++] = j;
            raw[fill[j]++] = i;
        }
    // sort and deduplicate each vertex's list (in parallel over vertices)
    std::vector<uint32_t> len(n);
    parallel_chunks(n, [&](size_t b, size_t e, unsigned) {
        for (size_t v = b; v < e; ++v) {
            auto first = raw.begin() + cnt[v], last = raw.begin() + cnt[v + 1];
            std::sort(first, last);
            len[v] = uint32_t(std::unique(first, last) - first);
        }
    });
    g.ptr.assign(size_t(n) + 1, 0);
    for (size_t v = 0; v < n; ++v) g.ptr[v + 1] = g.ptr[v] + len[v];
    g.adj.resize(g.ptr[n]);
    parallel_chunks(n, [&](size_t b, size_t e, unsigned) {
        for (size_t v = b; v < e; ++v)
            std::copy(raw.begin() + cnt[v], raw.begin() + cnt[v] + len[v], g.adj.begin() + g.ptr[v]);
    });
    return g;
}

// Breadth-first levels from `root` over unvisited vertices (mark[] != stamp);
// returns the vertices of the last level and the number of levels.
uint32_t bfs_last_level(const Graph& g, uint32_t root, std::vector<uint32_t>& mark, uint32_t stamp,
                        std::vector<uint32_t>& queue, std::vector<uint32_t>* last) {
    queue.clear();
    queue.push_back(root);
    mark[root] = stamp;
    size_t head = 0;
    uint32_t levels = 0;
    while (head < queue.size()) {
        const size_t level_end = queue.size();
        last->assign(queue.begin() + head, queue.begin() + level_end);
        ++levels;
        for (; head < level_end; ++head) {
            const uint32_t v = queue[head];
            for (uint64_t p = g.ptr[v]; p < g.ptr[v + 1]; ++p) {
                const uint32_t w = g.adj[p];
                if (mark[w] != stamp) {
                    mark[w] = stamp;
                    queue.push_back(w);
                }
            }
        }
    }
    return levels;
}

uint64_t bandwidth_of(const accspmm_csr_t* a, const uint32_t* inv) {
    uint64_t bw = 0;
    for (uint32_t i = 0; i < a->rows; ++i)
        for (uint32_t p = a->row_ptr[i]; p < a->row_ptr[i + 1]; ++p) {
            const uint64_t r = inv ? inv[i] : i, c = inv ? inv[a->col_idx[p]] : a->col_idx[p];
            bw = std::max(bw, r > c ? r - c : c - r);
        }
    return bw;
}

}  // namespace

int reorder_rcm_host(const accspmm_csr_t* a, uint32_t* perm, uint64_t* bw_before, uint64_t* bw_after) {
    if (a->space != ACCSPMM_HOST) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "the CSR must be in host memory");
    if (a->rows != a->cols) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "reordering needs a square matrix");
    const uint32_t n = a->rows;
    for (uint32_t p = 0; p < a->nnz; ++p)
        if (a->col_idx[p] >= n) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "column index out of range");
    const Graph g = symmetrise(a);
    // vertices by (degree, index): component roots are tried in this order
    std::vector<uint32_t> by_degree(n);
    std::iota(by_degree.begin(), by_degree.end(), 0u);
    std::stable_sort(by_degree.begin(), by_degree.end(),
                     [&](uint32_t x, uint32_t y) { return g.degree(x) < g.degree(y); });
    std::vector<uint32_t> mark(n, 0), queue, last;
    queue.reserve(n);
    std::vector<char> placed(n, 0);
    std::vector<uint32_t> order;
    order.reserve(n);
    std::vector<uint32_t> nb;
    uint32_t stamp = 0;
    for (uint32_t root0 : by_degree) {
        if (placed[root0]) continue;
        // pseudo-peripheral root: move to a minimum-degree vertex of the
        // last BFS level while that lengthens the level structure
        uint32_t root = root0;
        uint32_t levels = bfs_last_level(g, root, mark, ++stamp, queue, &last);
        for (int iter = 0; iter < 4; ++iter) {
            uint32_t cand = last[0];
            for (uint32_t v : last)
                if (g.degree(v) < g.degree(cand)) cand = v;
            const uint32_t l2 = bfs_last_level(g, cand, mark, ++stamp, queue, &last);
            if (l2 <= levels) break;
            root = cand;
            levels = l2;
        }
        // Cuthill-McKee from the root: neighbours in increasing degree
        const size_t begin = order.size();
        order.push_back(root);
        placed[root] = 1;
        for (size_t head = begin; head < order.size(); ++head) {
            const uint32_t v = order[head];
            nb.clear();
            for (uint64_t p = g.ptr[v]; p < g.ptr[v + 1]; ++p)
                if (!placed[g.adj[p]]) {
                    placed[g.adj[p]] = 1;
                    nb.push_back(g.adj[p]);
                }
            std::stable_sort(nb.begin(), nb.end(),
                             [&](uint32_t x, uint32_t y) { return g.degree(x) < g.degree(y); });
            order.insert(order.end(), nb.begin(), nb.end());
        }
    }
    // reversed
    for (uint32_t i = 0; i < n; ++i) perm[i] = order[n - 1 - i];
    if (bw_before) *bw_before = bandwidth_of(a, nullptr);
    if (bw_after) {
        std::vector<uint32_t> inv(n);
        for (uint32_t i = 0; i < n; ++i) inv[perm[i]] = i;
        *bw_after = bandwidth_of(a, inv.data());
    }
    return ACCSPMM_SUCCESS;
}

int csr_permute_host(const accspmm_csr_t* a, const uint32_t* perm, accspmm_csr_t* out) {
    if (a->space != ACCSPMM_HOST) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "the CSR must be in host memory");
    if (a->rows != a->cols) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "permuting needs a square matrix");
    const uint32_t n = a->rows;
    std::vector<uint32_t> inv(n, kPad);
    for (uint32_t i = 0; i < n; ++i) {
        if (perm[i] >= n || inv[perm[i]] != kPad) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "perm is not a permutation");
        inv[perm[i]] = i;
    }
    accspmm_csr_t c;
    std::memset(&c, 0, sizeof c);
    c.rows = c.cols = n;
    c.nnz = a->nnz;
    c.space = ACCSPMM_HOST;
    c.owned = 1;
    c.row_ptr = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * (size_t(n) + 1)));
    c.col_idx = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * (a->nnz ? a->nnz : 1)));
    c.data = static_cast<float*>(std::malloc(sizeof(float) * (a->nnz ? a->nnz : 1)));
    if (!c.row_ptr || !c.col_idx || !c.data) {
        accspmm_csr_destroy(&c);
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation failed");
    }
    c.row_ptr[0] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t r = perm[i];
        c.row_ptr[i + 1] = c.row_ptr[i] + (a->row_ptr[r + 1] - a->row_ptr[r]);
    }
    // each new row: the old row's entries with renumbered columns, sorted by
    // new column (stable, so duplicate entries keep their order)
    parallel_chunks(n, [&](size_t b, size_t e, unsigned) {
        std::vector<std::pair<uint32_t, uint32_t>> tmp;
        for (size_t i = b; i < e; ++i) {
            const uint32_t r = perm[i], p0 = a->row_ptr[r], len = a->row_ptr[r + 1] - p0;
            tmp.resize(len);
            for (uint32_t k = 0; k < len; ++k) tmp[k] = {inv[a->col_idx[p0 + k]], p0 + k};
            std::stable_sort(tmp.begin(), tmp.end(),
                             [](const std::pair<uint32_t, uint32_t>& x, const std::pair<uint32_t, uint32_t>& y) {
                                 return x.first < y.first;
                             });
            const uint32_t q0 = c.row_ptr[i];
            for (uint32_t k = 0; k < len; ++k) {
                c.col_idx[q0 + k] = tmp[k].first;
                c.data[q0 + k] = a->data[tmp[k].second];
            }
        }
    }, 1024);
    *out = c;
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
