// spmm_batch.cu -- many METCF matrices of different sizes and feature widths
// in one persistent launch.
//
// A batch is a table of per-matrix descriptors in device memory.  Every
// matrix is cut into the same work items (window block, feature slice) as a
// one-matrix launch -- the window-block size comes from the same chooser -- so
// each item's arithmetic, and therefore each result, is bit-identical to the
// matrix's own accspmm_spmm_tf32 launch.  Items are numbered largest matrix
// first; resident CTAs take items from an atomic counter until none are
// left, so uneven matrices share the GPU without a tail of idle SMs.  TF32
// matrices with K > 64 form a second group launched in 128-column slices
// with the rolling tile ring, their one-matrix default shape; a plan packs the
// B that the one-matrix rule packs (TF32, at least 4 MiB, K > 48) to 2.5-byte
// TF32 rows into buffers it owns, with one launch over all of them before the
// groups run, and their items read the packed rows (bit-identical).
// A plan can be captured into a CUDA graph (counter reset + launch) and
// replayed.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <numeric>
#include <vector>

#include "common.hpp"
#include "device_util.cuh"
#include "spmm_batch.hpp"
#include "spmm_common.cuh"
#include "spmm_direct.cuh"
#include "options.hpp"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

constexpr int kNW = kDirectNW;

// Work items of one launch: descriptors sorted by item0 (first item).
__device__ __forceinline__ uint32_t find_desc(const BatchDesc* __restrict__ d, uint32_t n,
                                              uint32_t item) {
    uint32_t lo = 0, hi = n;  // last desc with item0 <= item
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (d[mid].item0 <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// U tiles per gather batch and MINB resident CTAs per SM, as in the
// one-matrix register-direct kernel's default shape.  PK: every item has a
// packed B and runs the packed-B loop of the one-matrix packed kernel (with
// the L2 prefetch when K spans an odd number of 128-column slices, the
// one-matrix default); otherwise the fp32 loop.
template <int FS, int PREC, int U, int MINB, bool ROLL, bool PK = false>
__global__ void __launch_bounds__(kNW * 32, MINB)
spmm_batch_kernel(const BatchDesc* __restrict__ desc, uint32_t n_desc, uint32_t total_items,
                  uint32_t* __restrict__ counter) {
    extern __shared__ __align__(16) float smem[];
    float* part = smem;  // [2 kNW][8][FS]
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * kNW * 8 * FS);
    __shared__ SpmmArgs s_args;
    __shared__ uint32_t s_item, s_wbk, s_slice;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t item = atomicAdd(counter, 1u);
            s_item = item;
            if (item < total_items) {
                const uint32_t di = find_desc(desc, n_desc, item);
                const BatchDesc& d = desc[di];
                const uint32_t local = item - d.item0;
                s_args = SpmmArgs{d.rwo, d.tc_offset, d.bits, d.a2b, d.vals, d.B, d.C, d.W, d.cols,
                                  d.K, d.wb, d.n_slices, d.n_wblocks, 0, 0, nullptr, 0, nullptr,
                                  PK ? d.bp : nullptr, PK ? d.bpitch : 0u};
                s_wbk = local / d.n_slices;
                s_slice = local - s_wbk * d.n_slices;
            }
        }
        __syncthreads();
        if (s_item >= total_items) break;
        Block<FS, kNW> blk;
        blk.init_item(s_args, s_wbk, s_slice, s_rwo, part);
        if constexpr (PK && FS == 128) {
            if (s_args.n_slices & 1u) direct_item_packed<FS, U, kNW, true>(s_args, blk);
            else direct_item_packed<FS, U, kNW, false>(s_args, blk);
        } else if constexpr (PK) {
            direct_item_packed<FS, U, kNW, false>(s_args, blk);
        } else {
            direct_item<FS, PREC, U, false, kNW, ROLL>(s_args, blk);
        }
        __syncthreads();  // s_args, s_rwo and the slots are reused by the next item
    }
}

template <int FS, int PREC, bool ROLL, bool PK = false>
int launch_batch_t(const BatchDesc* d_desc, uint32_t n_desc, uint32_t total_items,
                   uint32_t max_wb, uint32_t* d_counter, cudaStream_t s) {
    // 128-column slices: 2 CTAs per SM with the one-matrix kernel's batch;
    // narrower slices: 3 CTAs per SM with half that batch
    constexpr int kMinB = FS == 128 ? 2 : 3;
    constexpr int kU = FS == 128 ? DirectBatch<FS>::U : (DirectBatch<FS>::U + 1) / 2;
    const size_t smem = size_t(2 * kNW * 8 * FS) * 4 + size_t(max_wb + 1) * 4;
    static unsigned attr_set = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_batch_kernel<FS, PREC, kU, kMinB, ROLL, PK>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set |= 1u << dev;
    }
    if (smem > 100 * 1024) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "window block too large for a batch");
    const uint32_t grid = std::min<uint32_t>(total_items, uint32_t(sm_count()) * kMinB);
    if (grid == 0) return ACCSPMM_SUCCESS;
    spmm_batch_kernel<FS, PREC, kU, kMinB, ROLL, PK><<<grid, kNW * 32, smem, s>>>(d_desc, n_desc, total_items, d_counter);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

// One matrix's B for the batched packing launch.
struct PackDesc {
    const float4* B;
    uint8_t* P;        // packed rows, then the zero row
    uint32_t K, pitch;
    uint32_t fs;       // slice width of the packed layout: 128 or 64
    uint64_t start;    // first float4 of this B in the launch's numbering
    uint64_t n4;       // float4s of this B
};

// Packs every listed B (pack_tf32_put layout) and writes each zero row; one
// float4 of B per thread and step, read once with a streaming load.  The
// grid walks the B one after another (each block strides through B j, then
// B j + 1), so no thread searches for its matrix.
__global__ void pack_tf32_batch_kernel(const PackDesc* __restrict__ d, uint32_t n, uint64_t total) {
    (void)total;
    for (uint32_t j = blockIdx.x; j < n; j += gridDim.x) {
        uint8_t* zero_row = d[j].P + (d[j].n4 / (d[j].K / 4)) * d[j].pitch;
        for (uint32_t t = threadIdx.x; t < d[j].pitch / 8; t += blockDim.x)
            reinterpret_cast<uint2*>(zero_row)[t] = make_uint2(0u, 0u);
    }
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    // thread t's first index in B j continues where its strides through the
    // previous B ended, so every thread's work stays within one pass of the
    // grid over the concatenated float4s
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (uint32_t j = 0; j < n; ++j) {
        const PackDesc x = d[j];
        const uint32_t k4 = x.K / 4;
        for (; i < x.start + x.n4; i += stride) {
            const uint64_t local = i - x.start;
            const uint64_t row = local / k4;
            const uint32_t c = uint32_t(local - row * k4) * 4;
            if (x.fs == 64) pack_tf32_put<64>(x.P + row * x.pitch, c, __ldcs(x.B + local));
            else pack_tf32_put<128>(x.P + row * x.pitch, c, __ldcs(x.B + local));
        }
    }
}

}  // namespace

// slice width of the narrow group: the one-matrix default (32 columns for
// K <= 32, else 64)
int batch_fs_for(uint32_t max_k) { return max_k <= 32 ? 32 : 64; }

bool batch_item_is_wide(uint32_t K, int precision) {
#ifdef ACCSPMM_LAB
    // measurement: ACCSPMM_BATCH_WIDE=0 runs wide items in the narrow group
    if (lab_env("ACCSPMM_BATCH_WIDE", 1) == 0) return false;
#endif
    return precision == ACCSPMM_PREC_TF32 && K > 64;
}

int launch_batch(const BatchDesc* d_desc, uint32_t n_desc, uint32_t total_items, uint32_t max_wb,
                 uint32_t* d_counter, int fs, int precision, cudaStream_t s, bool packed) {
    ACC_CUDA(cudaMemsetAsync(d_counter, 0, 4, s));
    const bool x3 = precision == ACCSPMM_PREC_3XTF32;
    // the rolling tile ring spills in the persistent kernel (24 bytes) and
    // measured 6 % slower on 128 power-law graphs: off (the measurement build
    // turns it on with ACCSPMM_BATCH_ROLL=1)
#ifdef ACCSPMM_LAB
    const bool roll = lab_env("ACCSPMM_BATCH_ROLL", 0) == 1;
#else
    const bool roll = false;
#endif
    if (fs == 128) {
        // wide TF32 items: 128-column slices with the rolling tile ring, the
        // one-matrix default for K > 64
        if (x3) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "128-column batch slices are TF32 only");
        if (packed)
            return launch_batch_t<128, ACCSPMM_PREC_TF32, true, true>(d_desc, n_desc, total_items, max_wb, d_counter, s);
        return launch_batch_t<128, ACCSPMM_PREC_TF32, true>(d_desc, n_desc, total_items, max_wb, d_counter, s);
    }
    if (packed) {
        // narrow TF32 items over 160-byte packed slices of 64 columns
        if (fs != 64 || x3) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "packed narrow batch slices are 64-column TF32");
        return launch_batch_t<64, ACCSPMM_PREC_TF32, false, true>(d_desc, n_desc, total_items, max_wb, d_counter, s);
    }
    switch (fs) {
        case 32: return x3 ? launch_batch_t<32, ACCSPMM_PREC_3XTF32, false>(d_desc, n_desc, total_items, max_wb, d_counter, s)
                           : launch_batch_t<32, ACCSPMM_PREC_TF32, false>(d_desc, n_desc, total_items, max_wb, d_counter, s);
        default:
            if (roll)
                return x3 ? launch_batch_t<64, ACCSPMM_PREC_3XTF32, true>(d_desc, n_desc, total_items, max_wb, d_counter, s)
                          : launch_batch_t<64, ACCSPMM_PREC_TF32, true>(d_desc, n_desc, total_items, max_wb, d_counter, s);
            return x3 ? launch_batch_t<64, ACCSPMM_PREC_3XTF32, false>(d_desc, n_desc, total_items, max_wb, d_counter, s)
                      : launch_batch_t<64, ACCSPMM_PREC_TF32, false>(d_desc, n_desc, total_items, max_wb, d_counter, s);
    }
}

int make_batch_descs(const BatchInput* in, uint32_t n, int fs, int precision,
                     std::vector<BatchDesc>* out, uint32_t* total_items, uint32_t* max_wb) {
    std::vector<BatchDesc> d(n);
    std::vector<uint64_t> work(n);
    for (uint32_t i = 0; i < n; ++i) {
        const BatchInput& x = in[i];
        if (x.K == 0 || x.K % 4) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "item %u: K=%u must be a positive multiple of 4", i, x.K);
        if (!x.B || !x.C || ((reinterpret_cast<uintptr_t>(x.B) | reinterpret_cast<uintptr_t>(x.C)) & 15u))
            ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "item %u: B and C must be 16-byte aligned device pointers", i);
        const uint32_t wb = window_block_for(x.w_cfg, x.T, x.K, precision);
        const uint32_t slices = (x.K + uint32_t(fs) - 1) / uint32_t(fs);
        d[i] = BatchDesc{x.rwo, x.tc_offset, x.bits, x.a2b, x.vals, x.B, x.C, x.W, x.cols, x.K,
                         wb, slices, (x.W + wb - 1) / wb, 0, 0};
        work[i] = uint64_t(x.T + x.W) * slices;
    }
    // largest matrix first
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return work[a] > work[b]; });
    out->clear();
    uint64_t items = 0;
    uint32_t mwb = 1;
    for (uint32_t k = 0; k < n; ++k) {
        BatchDesc x = d[order[k]];
        if (x.W == 0) continue;
        x.item0 = uint32_t(items);
        x.index = order[k];
        items += uint64_t(x.n_wblocks) * x.n_slices;
        mwb = std::max(mwb, x.wb);
        out->push_back(x);
    }
    if (items > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "too many work items in a batch");
    *total_items = uint32_t(items);
    *max_wb = mwb;
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm

// ---------------------------------------------------------------------------
// C ABI: batch plans
// ---------------------------------------------------------------------------
using namespace accspmm;

// One persistent launch of a plan: the items of one slice-width class.
struct BatchGroup {
    int fs = 64;
    bool packed = false;  // every item reads a packed B
    uint32_t n_desc = 0, total_items = 0, max_wb = 1;
    BatchDesc* d_desc = nullptr;
    uint32_t* d_counter = nullptr;
};

// A plan: TF32 items with K > 64 run in 128-column slices with the tile ring
// (the one-matrix default for them), the others in the narrow shape; in each,
// the items whose B the one-matrix rule packs form a group of their own that
// reads packed copies (128- or 64-column slices, written by one packing
// launch at the start of each run); one persistent launch per non-empty
// group, wide groups first.
struct accspmm_batch {
    int device = 0;
    int precision = ACCSPMM_PREC_TF32;
    std::vector<BatchGroup> groups;
    // packed copies of the packed groups' B (owned, one buffer per group),
    // all written by one launch at the start of a run
    std::vector<void*> packed_bufs;
    std::vector<PackDesc> pack_host;
    PackDesc* d_pack = nullptr;
    uint32_t n_pack = 0;
    uint64_t pack_total = 0;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
};

static void free_groups(accspmm_batch* b) {
    for (auto& g : b->groups) {
        cudaFree(g.d_desc);
        cudaFree(g.d_counter);
    }
    b->groups.clear();
    for (void* p : b->packed_bufs) cudaFree(p);
    b->packed_bufs.clear();
    b->pack_host.clear();
    cudaFree(b->d_pack);
    b->d_pack = nullptr;
    b->n_pack = 0;
    b->pack_total = 0;
}

// Whether an item's B is packed: the one-matrix rule -- TF32, a B of at
// least 4 MiB, K > 64 (128-column slices) or 48 < K <= 64 (64-column slices),
// or as ACCSPMM_OPT_PACK says (1: every TF32 item with K > 32).
static bool batch_item_packs(uint32_t cols, uint32_t K, int precision) {
    if (precision != ACCSPMM_PREC_TF32 || cols == 0 || K <= 32) return false;
    const int pk = option(ACCSPMM_OPT_PACK);
    const uint64_t b_bytes = uint64_t(cols) * K * 4;
    return pk > 0 || (pk < 0 && K > 48 && b_bytes >= (uint64_t(4) << 20));
}

// Packed copies (FS-column layout) of the B of every item in d, in one buffer
// owned by the plan; points the descriptors at them and lists them for the
// packing launch (upload_packing puts the list on the device).
static int plan_packing(accspmm_batch* b, std::vector<BatchDesc>* d, uint32_t fs) {
    std::vector<size_t> off(d->size(), SIZE_MAX);
    size_t bytes = 0;
    for (size_t i = 0; i < d->size(); ++i) {
        const BatchDesc& x = (*d)[i];
        if (x.cols == 0) continue;
        off[i] = bytes;
        const size_t pitch = size_t(fs * 5 / 2) * ((x.K + fs - 1) / fs);
        bytes += ((size_t(x.cols) + 1) * pitch + 64 + 255) / 256 * 256;
    }
    if (bytes == 0) return ACCSPMM_SUCCESS;
    void* buf = nullptr;
    if (cudaMalloc(&buf, bytes) != cudaSuccess)
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "device allocation of the packed B copies (%zu bytes) failed", bytes);
    b->packed_bufs.push_back(buf);
    uint8_t* base = static_cast<uint8_t*>(buf);
    for (size_t i = 0; i < d->size(); ++i) {
        if (off[i] == SIZE_MAX) continue;
        BatchDesc& x = (*d)[i];
        x.bp = base + off[i];
        x.bpitch = (fs * 5 / 2) * ((x.K + fs - 1) / fs);
        const uint64_t n4 = uint64_t(x.cols) * (x.K / 4);
        b->pack_host.push_back(PackDesc{reinterpret_cast<const float4*>(x.B), base + off[i], x.K, x.bpitch, fs,
                                        b->pack_total, n4});
        b->pack_total += n4;
    }
    return ACCSPMM_SUCCESS;
}

static int upload_packing(accspmm_batch* b) {
    if (b->pack_host.empty()) return ACCSPMM_SUCCESS;
    const size_t bytes = sizeof(PackDesc) * b->pack_host.size();
    if (cudaMalloc(&b->d_pack, bytes) != cudaSuccess ||
        cudaMemcpy(b->d_pack, b->pack_host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "device table of the packed B copies failed");
    b->n_pack = uint32_t(b->pack_host.size());
    return ACCSPMM_SUCCESS;
}

extern "C" {

int accspmm_batch_create(const accspmm_batch_item_t* items, uint32_t n, int32_t precision,
                         accspmm_batch_t** out) {
    clear_error();
    if (!out || (n && !items)) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (precision != ACCSPMM_PREC_TF32 && precision != ACCSPMM_PREC_3XTF32)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    *out = nullptr;
    std::vector<BatchInput> in(n);
    for (uint32_t i = 0; i < n; ++i) {
        const accspmm_metcf_t* m = items[i].metcf;
        if (!m || m->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "item %u: METCF must be on the device", i);
        in[i] = BatchInput{m->row_window_offset, m->tc_offset, m->tc_local_bit, m->sparse_a2b, m->data,
                           items[i].B, items[i].C, m->num_windows, m->num_windows, m->num_tiles,
                           m->cols, items[i].K};
    }
    auto* b = new accspmm_batch();
    cudaGetDevice(&b->device);
    b->precision = precision;
    // split by class -- wide with packed B, wide reading fp32 B, narrow with
    // packed B (64-column slices), narrow reading fp32 B -- keeping each
    // item's position for its index
    std::vector<BatchInput> cls[4];
    std::vector<uint32_t> pos[4];
    uint32_t narrow_k = 4;
    for (uint32_t i = 0; i < n; ++i) {
        const bool packs = batch_item_packs(in[i].cols, in[i].K, precision);
        const int c = batch_item_is_wide(in[i].K, precision) ? (packs ? 0 : 1) : (packs ? 2 : 3);
        cls[c].push_back(in[i]);
        pos[c].push_back(i);
        if (c == 3) narrow_k = std::max(narrow_k, in[i].K);
    }
    for (int c = 0; c < 4; ++c) {
        if (cls[c].empty()) continue;
        BatchGroup g;
        g.fs = c < 2 ? 128 : c == 2 ? 64 : batch_fs_for(narrow_k);
        g.packed = c == 0 || c == 2;
        std::vector<BatchDesc> d;
        int st = make_batch_descs(cls[c].data(), uint32_t(cls[c].size()), g.fs, precision, &d,
                                  &g.total_items, &g.max_wb);
        if (st) {
            free_groups(b);
            delete b;
            return st;
        }
        for (auto& x : d) x.index = pos[c][x.index];
        if (g.packed && (st = plan_packing(b, &d, uint32_t(g.fs)))) {
            free_groups(b);
            delete b;
            return st;
        }
        g.n_desc = uint32_t(d.size());
        if (cudaMalloc(&g.d_desc, sizeof(BatchDesc) * std::max<size_t>(1, d.size())) != cudaSuccess ||
            cudaMalloc(&g.d_counter, 4) != cudaSuccess) {
            cudaFree(g.d_desc);
            free_groups(b);
            delete b;
            ACC_FAIL(ACCSPMM_ERROR_ALLOC, "device allocation of the batch table failed");
        }
        b->groups.push_back(g);
        if (!d.empty() &&
            cudaMemcpy(g.d_desc, d.data(), sizeof(BatchDesc) * d.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            free_groups(b);
            delete b;
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "copy of the batch table failed");
        }
    }
    if (const int st = upload_packing(b)) {
        free_groups(b);
        delete b;
        return st;
    }
    *out = b;
    return ACCSPMM_SUCCESS;
}

int accspmm_batch_run(accspmm_batch_t* b, void* stream) {
    clear_error();
    if (!b) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null batch");
    if (b->n_pack) {
        // this run's B values, packed before the wide group reads them
        const unsigned blocks = unsigned(std::min<uint64_t>((b->pack_total + 255) / 256 + 1,
                                                            uint64_t(sm_count()) * 16));
        pack_tf32_batch_kernel<<<blocks, 256, 0, as_stream(stream)>>>(b->d_pack, b->n_pack, b->pack_total);
        ACC_LAUNCH_CHECK();
    }
    for (const auto& g : b->groups) {
        if (g.total_items == 0) continue;
        const int st = launch_batch(g.d_desc, g.n_desc, g.total_items, g.max_wb, g.d_counter, g.fs,
                                    b->precision, as_stream(stream), g.packed);
        if (st) return st;
    }
    return ACCSPMM_SUCCESS;
}

int accspmm_batch_capture(accspmm_batch_t* b, void* stream) {
    clear_error();
    if (!b) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null batch");
    cudaStream_t s = as_stream(stream);
    if (!s) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "graph capture needs a non-default stream");
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
    }
    // make sure the kernels' attributes are set outside the capture
    ACC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int st = accspmm_batch_run(b, stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        ACC_FAIL(ACCSPMM_ERROR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    }
    b->graph = g;
    return ACCSPMM_SUCCESS;
}

int accspmm_batch_launch_graph(accspmm_batch_t* b, void* stream) {
    clear_error();
    if (!b || !b->exec) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "batch has no captured graph");
    ACC_CUDA(cudaGraphLaunch(b->exec, as_stream(stream)));
    return ACCSPMM_SUCCESS;
}

int accspmm_batch_info(const accspmm_batch_t* b, uint32_t* n_items, uint32_t* work_items,
                       uint32_t* slice_width) {
    clear_error();
    if (!b) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null batch");
    uint32_t n = 0, w = 0, fs = 0;
    for (const auto& g : b->groups) {
        n += g.n_desc;
        w += g.total_items;
        fs = std::max<uint32_t>(fs, uint32_t(g.fs));
    }
    if (n_items) *n_items = n;
    if (work_items) *work_items = w;
    if (slice_width) *slice_width = fs;
    return ACCSPMM_SUCCESS;
}

void accspmm_batch_destroy(accspmm_batch_t* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    free_groups(b);
    delete b;
}

}  // extern "C"
