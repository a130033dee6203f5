// dense_gemm.cu -- XW = H W for the graph-convolution layer, on the fifth-
// generation tensor cores: tcgen05.mma kind::tf32 with the accumulator in
// tensor memory, operands staged in shared memory by the tensor-map copy
// engine (cp.async.bulk.tensor, 128-byte swizzle).  No counterpart in the
// reference, which multiplies A by a constant B only (src/mma_tf32.cu:185-243);
// this is the dense product of accspmm_gcn_layer and accspmm_dense_matmul.
//
// Shapes: H is n x k_in, W is k_in x k_out, both row-major fp32, n large
// (graph rows) and k_in, k_out feature widths.  Work is cut into 128-row by
// NT-column tiles of XW (NT = k_out rounded up to 16, at most 256 in TF32 and
// 128 in 3xTF32; wider outputs take several column tiles); k_in is walked in
// blocks of 32 through a ring of shared-memory stages, each holding the
// 128 x 32 block of H and the NT x 32 block of W^T (W transposed and rounded
// to TF32 once per call into a K-major pool buffer, so that both operands are
// K-major), copied by tensor-map loads.  The H block is rounded to TF32 in
// place (cvt.rna, the rounding of the SpMM's operands) before the MMAs read
// it; the MMAs are tcgen05.mma with K = 8, four per block.
//
// TF32 (dense_gemm_tf32_ws_kernel): persistent and warp-specialised -- copies,
// rounding, MMAs into two alternating TMEM accumulators, and stores through
// shared memory and tensor-map stores all overlap (described at the kernel).
// 3xTF32 (dense_gemm_3xtf32_ws_kernel): the same structure; H and W are split
// into hi + lo TF32 parts, three products per K step (hi*hi, hi*lo, lo*hi),
// and every k-block's partial is summed in FP32 registers (described at the
// kernel).
//
// Every wait is bounded (2 s of %globaltimer); a wait that runs out raises
// a bit in the status word that accspmm_device_status reports, the CTA waits
// (bounded) for its copies in flight and its MMAs, stores nothing, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "accspmm.h"
#include "common.hpp"
#include "device_util.cuh"
#include "mbarrier.cuh"
#include "spmm_common.cuh"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

__device__ unsigned int g_gemm_status = 0;

constexpr int kBM = 128;       // rows of H per CTA: the MMA's M
constexpr int kBK = 32;        // k per stage: one 128-byte swizzle row of fp32
constexpr uint32_t kATileBytes = kBM * kBK * 4;  // 16 KB

// Shared-memory matrix descriptor of a K-major operand tile written by a TMA
// copy with 128-byte swizzle: rows of 128 bytes (32 fp32 along k), 8-row
// groups 1024 bytes apart (stride byte offset), tile base 1024-byte aligned.
// Fields: start address >> 4 (bits 0-13), leading byte offset >> 4 (16-29;
// not used by swizzled K-major layouts whose MMA k fits in one row), stride
// byte offset >> 4 (32-45), descriptor version 1 (46-47), base offset 0
// (49-51), swizzle mode 2 = 128 B (61-63).
__device__ __forceinline__ uint64_t kmajor_sw128_desc(uint32_t saddr) {
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(1) << 16) | (uint64_t(1024 >> 4) << 32) |
           (uint64_t(1) << 46) | (uint64_t(2) << 61);
}

// Instruction descriptor of tcgen05.mma kind::tf32: D fp32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 (bits 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t idesc_tf32(uint32_t m, uint32_t n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The barrier gets one arrival once every MMA this thread issued so far is done.
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// TF32: a persistent, warp-specialised kernel.  Each CTA walks work items
// (128-row x NT-column tiles of XW, column tile fastest) with five roles:
//   warp 0, one lane   -- copies: the H and W^T blocks of every item into a
//                         ring of S stages (tensor-map loads, "full" barriers);
//   warps 2-5          -- round the H block of each landed stage to TF32 in
//                         place (cvt.rna) and mark it ready ("conv");
//   warp 1, one lane   -- MMAs: four K = 8 tcgen05.mma per block into one of
//                         two tensor-memory accumulators (items alternate),
//                         committing each stage back to the copier ("empty")
//                         and each finished accumulator to the store warps
//                         ("tfull");
//   warps 6-9          -- store: each reads its 32 TMEM lanes (rows) of the
//                         finished accumulator 32 columns at a time, writes
//                         them to a swizzled 4 KB staging buffer and stores
//                         it with a tensor-map store, then frees the
//                         accumulator ("tempty").
// So the copies of the next blocks, the rounding, the MMAs of item i + 1 and
// the stores of item i all run at once.  Every wait is bounded: a wait that
// runs out sets an abort flag that ends every role's loop, and raises the
// status bit; each role then waits (bounded) for its own asynchronous work
// and the CTA frees its tensor memory.

constexpr int kWsThreads = 320;       // ten warps
constexpr uint32_t kStageOut = 4096;  // one store warp's staging buffer: 32 rows x 32 fp32

struct WsParams {
    uint32_t n, k_out;
    uint32_t kblocks;    // ceil(kp / 32)
    uint32_t nt;         // output columns per item (multiple of 16, <= 256)
    uint32_t n_tiles;    // column tiles: ceil(k_out / nt)
    uint32_t items;      // ceil(n / 128) * n_tiles
    uint32_t stages;
    uint32_t stage_bytes;
    uint32_t acc_stride;  // TMEM columns between the two accumulators (power of two >= max(32, nt))
    uint32_t tmem_cols;   // 2 * acc_stride
};

__device__ __forceinline__ bool wait_or_abort(uint32_t bar, uint32_t parity, volatile int* abort) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
        if (global_ns() - t0 > kWaitLimitNs) {
            *abort = 1;
            atomicOr(&g_gemm_status, 1u);
            return false;
        }
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* tm, int x, int y, uint32_t src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(tm)),
                 "r"(x), "r"(y), "r"(src)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__global__ void __launch_bounds__(kWsThreads, 1)
    dense_gemm_tf32_ws_kernel(const __grid_constant__ CUtensorMap tm_h, const __grid_constant__ CUtensorMap tm_w,
                              const __grid_constant__ CUtensorMap tm_out, const WsParams p) {
    extern __shared__ uint8_t dyn_smem[];
    // full[8], conv[8], empty[8], tfull[2], tempty[2], done
    __shared__ __align__(8) uint64_t bars[3 * 8 + 5];
    __shared__ uint32_t s_tmem;
    __shared__ volatile int s_abort;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t S = p.stages;
    const uint32_t base = (smem_addr(dyn_smem) + 1023u) & ~1023u;
    uint8_t* gbase = dyn_smem + (base - smem_addr(dyn_smem));
    const uint32_t out_base = base + S * p.stage_bytes;  // 4 store warps x 2 buffers x 4 KB
    auto full = [&](uint32_t s) { return smem_addr(&bars[s]); };
    auto conv = [&](uint32_t s) { return smem_addr(&bars[8 + s]); };
    auto empty = [&](uint32_t s) { return smem_addr(&bars[16 + s]); };
    auto tfull = [&](uint32_t b) { return smem_addr(&bars[24 + b]); };
    auto tempty = [&](uint32_t b) { return smem_addr(&bars[26 + b]); };
    const uint32_t done = smem_addr(&bars[28]);
    const uint32_t b_off = kATileBytes;
    const uint32_t tx_bytes = kATileBytes + p.nt * 128u;

    if (tid == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            mbar_init(full(s), 1);
            mbar_init(conv(s), 4);
            mbar_init(empty(s), 1);
        }
        for (uint32_t b = 0; b < 2; ++b) {
            mbar_init(tfull(b), 1);
            mbar_init(tempty(b), 4);
        }
        mbar_init(done, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                     "r"(p.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    if (warp == 0) {
        // copier
        if (lane == 0) {
            uint32_t it = 0;
            bool go = true;
            for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x) {
                const int m0 = int(item / p.n_tiles) * kBM, n0 = int((item % p.n_tiles) * p.nt);
                for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                    const uint32_t s = it % S, use = it / S;
                    if (use > 0 && !wait_or_abort(empty(s), (use - 1) & 1u, &s_abort)) {
                        go = false;
                        break;
                    }
                    const uint32_t st = base + s * p.stage_bytes;
                    mbar_expect_tx(full(s), tx_bytes);
                    tma_load_2d(st, &tm_h, int(kb * kBK), m0, full(s));
                    tma_load_2d(st + b_off, &tm_w, int(kb * kBK), n0, full(s));
                }
            }
            // the last S copies may still be in flight when the loop ended early
            const uint32_t first = it > S ? it - S : 0;
            for (uint32_t i = first; i < it; ++i) mbar_wait(full(i % S), (i / S) & 1u);
        }
    } else if (warp == 1) {
        // MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(kBM, p.nt);
            uint32_t it = 0, t = 0;
            bool go = true;
            for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x, ++t) {
                const uint32_t b = t & 1u, use_b = t >> 1;
                if (use_b > 0 && !wait_or_abort(tempty(b), (use_b - 1) & 1u, &s_abort)) break;
                tc_fence_after();
                const uint32_t d = tmem + b * p.acc_stride;
                for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                    const uint32_t s = it % S;
                    if (!wait_or_abort(conv(s), (it / S) & 1u, &s_abort)) {
                        go = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = base + s * p.stage_bytes;
#pragma unroll
                    for (uint32_t j = 0; j < kBK / 8; ++j)
                        umma_tf32(d, kmajor_sw128_desc(sa + j * 32), kmajor_sw128_desc(sa + b_off + j * 32), idesc,
                                  (kb > 0 || j > 0) ? 1u : 0u);
                    umma_commit(empty(s));
                }
                if (go) umma_commit(tfull(b));
            }
            // no MMA may still run when the tensor memory is freed
            umma_commit(done);
            mbar_wait(done, 0);
        }
    } else if (warp < 6) {
        // rounding: 128 threads, 8 float4 of each 16 KB H block
        const uint32_t ct = tid - 64;
        uint32_t it = 0;
        bool go = true;
        for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x) {
            for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                const uint32_t s = it % S;
                const bool landed = __all_sync(0xffffffffu, wait_or_abort(full(s), (it / S) & 1u, &s_abort));
                if (!landed) {
                    go = false;
                    break;
                }
                float4* ah = reinterpret_cast<float4*>(gbase + s * p.stage_bytes);
#pragma unroll
                for (int i = 0; i < int(kATileBytes / 16 / 128); ++i) {
                    const uint32_t idx = ct + uint32_t(i) * 128u;
                    const float4 x = ah[idx];
                    ah[idx] = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(conv(s));
            }
        }
    } else {
        // stores: warp w reads TMEM lanes 32 (w % 4) .. +31, i.e. rows m0 + 32 (w % 4) + lane
        const uint32_t q = warp & 3u;
        const uint32_t obuf = out_base + (warp - 6) * 2 * kStageOut;
        uint8_t* gobuf = gbase + (obuf - base);
        uint32_t t = 0, nst = 0;
        for (uint32_t item = blockIdx.x; item < p.items; item += gridDim.x, ++t) {
            const uint32_t b = t & 1u;
            const bool ready = __all_sync(0xffffffffu, wait_or_abort(tfull(b), (t >> 1) & 1u, &s_abort));
            if (!ready) break;
            tc_fence_after();
            const int m0 = int(item / p.n_tiles) * kBM, n0 = int((item % p.n_tiles) * p.nt);
            const uint32_t t_row = tmem + b * p.acc_stride + ((q * 32u) << 16);
            for (uint32_t c = 0; c * 32 < p.nt; ++c) {
                // chunks wholly past the matrix's rows or columns store nothing
                if (uint32_t(m0) + q * 32u >= p.n || uint32_t(n0) + c * 32u >= p.k_out) continue;
                ++nst;
                uint32_t r[32];
                tmem_ld32(t_row + c * 32, r);
                // the store that used this buffer two chunks ago has read it
                if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                __syncwarp();
                const uint32_t buf = (nst & 1u) * kStageOut;
                uint8_t* row = gobuf + buf + lane * 128u;
#pragma unroll
                for (uint32_t j = 0; j < 8; ++j)
                    *reinterpret_cast<uint4*>(row + ((j ^ (lane & 7u)) * 16u)) =
                        make_uint4(r[4 * j], r[4 * j + 1], r[4 * j + 2], r[4 * j + 3]);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) tma_store_2d(&tm_out, n0 + int(c * 32), m0 + int(q * 32), obuf + buf);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty(b));
        }
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// 3xTF32, persistent and warp-specialised: the TF32 kernel's structure with
// the operands split into hi + lo TF32 parts and a per-block drain of the
// accumulators.  Fourteen warps:
//   warp 0, one lane  -- copies: per k-block the 128 x 32 block of H and the
//                        NT x 32 blocks of W^T hi and lo ("full");
//   warps 2-5         -- split the H block in place: hi = rna(x) over x,
//                        lo = rna(x - hi) beside it ("conv");
//   warp 1, one lane  -- twelve MMAs per k-block into the region of its
//                        parity: hi*hi into 128 columns, lo*hi and hi*lo into
//                        the next 128 ("bfull"), freeing the stage ("empty");
//   warps 6-13        -- two per TMEM lane quarter, each for 64 of the tile's
//                        columns: add every block's main and correction
//                        partials to FP32 registers with round-to-nearest as
//                        soon as the block is done, free the region
//                        ("bempty"), and after the item's last block store the
//                        registers through shared memory and tensor-map
//                        stores.
// The tensor core accumulates only the four K = 8 steps of one block (its
// own accumulation over all of k_in is not round-to-nearest and gave 1.8e-6
// relative error at k_in = 256).

constexpr int kX3Threads = 448;  // fourteen warps

__global__ void __launch_bounds__(kX3Threads, 1)
    dense_gemm_3xtf32_ws_kernel(const __grid_constant__ CUtensorMap tm_h, const __grid_constant__ CUtensorMap tm_w,
                                const __grid_constant__ CUtensorMap tm_wlo, const __grid_constant__ CUtensorMap tm_out,
                                const WsParams p) {
    extern __shared__ uint8_t dyn_smem[];
    // full[4], conv[4], empty[4], bfull[2], bempty[2], done
    __shared__ __align__(8) uint64_t bars[3 * 4 + 5];
    __shared__ uint32_t s_tmem;
    __shared__ volatile int s_abort;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t S = p.stages;
    const uint32_t base = (smem_addr(dyn_smem) + 1023u) & ~1023u;
    uint8_t* gbase = dyn_smem + (base - smem_addr(dyn_smem));
    const uint32_t out_base = base + S * p.stage_bytes;  // 8 drain warps x 4 KB
    auto full = [&](uint32_t s) { return smem_addr(&bars[s]); };
    auto conv = [&](uint32_t s) { return smem_addr(&bars[4 + s]); };
    auto empty = [&](uint32_t s) { return smem_addr(&bars[8 + s]); };
    auto bfull = [&](uint32_t r) { return smem_addr(&bars[12 + r]); };
    auto bempty = [&](uint32_t r) { return smem_addr(&bars[14 + r]); };
    const uint32_t done = smem_addr(&bars[16]);
    // stage: [A hi 16 KB][A lo 16 KB][W^T hi nt x 128 B][W^T lo nt x 128 B]
    const uint32_t a_lo = kATileBytes, b_hi = 2 * kATileBytes, b_lo = b_hi + p.nt * 128u;
    const uint32_t tx_bytes = kATileBytes + 2u * p.nt * 128u;

    if (tid == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            mbar_init(full(s), 1);
            mbar_init(conv(s), 4);
            mbar_init(empty(s), 1);
        }
        for (uint32_t r = 0; r < 2; ++r) {
            mbar_init(bfull(r), 1);
            mbar_init(bempty(r), 8);
        }
        mbar_init(done, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                     "r"(512u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            bool go = true;
            for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x) {
                const int m0 = int(item / p.n_tiles) * kBM, n0 = int((item % p.n_tiles) * p.nt);
                for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                    const uint32_t s = it % S, use = it / S;
                    if (use > 0 && !wait_or_abort(empty(s), (use - 1) & 1u, &s_abort)) {
                        go = false;
                        break;
                    }
                    const uint32_t st = base + s * p.stage_bytes;
                    mbar_expect_tx(full(s), tx_bytes);
                    tma_load_2d(st, &tm_h, int(kb * kBK), m0, full(s));
                    tma_load_2d(st + b_hi, &tm_w, int(kb * kBK), n0, full(s));
                    tma_load_2d(st + b_lo, &tm_wlo, int(kb * kBK), n0, full(s));
                }
            }
            const uint32_t first = it > S ? it - S : 0;
            for (uint32_t i = first; i < it; ++i) mbar_wait(full(i % S), (i / S) & 1u);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(kBM, p.nt);
            uint32_t it = 0;  // k-blocks issued, over all items: block it uses region it & 1
            bool go = true;
            for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x) {
                for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                    const uint32_t s = it % S, r = it & 1u, use_r = it >> 1;
                    if (use_r > 0 && !wait_or_abort(bempty(r), (use_r - 1) & 1u, &s_abort)) {
                        go = false;
                        break;
                    }
                    if (!wait_or_abort(conv(s), (it / S) & 1u, &s_abort)) {
                        go = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = base + s * p.stage_bytes;
                    const uint32_t t_main = tmem + r * 256u;
#pragma unroll
                    for (uint32_t j = 0; j < kBK / 8; ++j) {
                        const uint64_t dah = kmajor_sw128_desc(sa + j * 32);
                        const uint64_t dal = kmajor_sw128_desc(sa + a_lo + j * 32);
                        const uint64_t dbh = kmajor_sw128_desc(sa + b_hi + j * 32);
                        const uint64_t dbl = kmajor_sw128_desc(sa + b_lo + j * 32);
                        umma_tf32(t_main, dah, dbh, idesc, j > 0 ? 1u : 0u);
                        umma_tf32(t_main + 128, dal, dbh, idesc, j > 0 ? 1u : 0u);
                        umma_tf32(t_main + 128, dah, dbl, idesc, 1u);
                    }
                    umma_commit(empty(s));
                    umma_commit(bfull(r));
                }
            }
            umma_commit(done);
            mbar_wait(done, 0);
        }
    } else if (warp < 6) {
        // split: 128 threads, 8 float4 of each 16 KB H block
        const uint32_t ct = tid - 64;
        uint32_t it = 0;
        bool go = true;
        for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x) {
            for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                const uint32_t s = it % S;
                if (!__all_sync(0xffffffffu, wait_or_abort(full(s), (it / S) & 1u, &s_abort))) {
                    go = false;
                    break;
                }
                float4* ah = reinterpret_cast<float4*>(gbase + s * p.stage_bytes);
                float4* al = reinterpret_cast<float4*>(gbase + s * p.stage_bytes + a_lo);
#pragma unroll
                for (int i = 0; i < int(kATileBytes / 16 / 128); ++i) {
                    const uint32_t idx = ct + uint32_t(i) * 128u;
                    const float4 x = ah[idx];
                    const float4 h = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
                    ah[idx] = h;
                    al[idx] = make_float4(tf32_hi(x.x - h.x), tf32_hi(x.y - h.y), tf32_hi(x.z - h.z),
                                          tf32_hi(x.w - h.w));
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(conv(s));
            }
        }
    } else {
        // drain and store: TMEM lanes 32 (w % 4) .. +31, columns 64 hc .. +63
        const uint32_t q = warp & 3u, hc = (warp - 6) >> 2;
        const uint32_t obuf = out_base + (warp - 6) * kStageOut;
        uint8_t* gobuf = gbase + (obuf - base);
        const uint32_t t_lane = (q * 32u) << 16;
        uint32_t it = 0;
        bool go = true;
        for (uint32_t item = blockIdx.x; go && item < p.items; item += gridDim.x) {
            const int m0 = int(item / p.n_tiles) * kBM, n0 = int((item % p.n_tiles) * p.nt);
            float acc[64];
#pragma unroll
            for (int i = 0; i < 64; ++i) acc[i] = 0.f;
            for (uint32_t kb = 0; kb < p.kblocks; ++kb, ++it) {
                const uint32_t r = it & 1u;
                if (!__all_sync(0xffffffffu, wait_or_abort(bfull(r), (it >> 1) & 1u, &s_abort))) {
                    go = false;
                    break;
                }
                tc_fence_after();
                const uint32_t t_main = tmem + r * 256u + t_lane + 64u * hc;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if (64u * hc + uint32_t(c) * 16u < p.nt) {
                        float v[16], w[16];
                        tmem_ld16(t_main + c * 16, v);
                        tmem_ld16(t_main + 128 + c * 16, w);
#pragma unroll
                        for (int i = 0; i < 16; ++i) acc[c * 16 + i] += v[i] + w[i];
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bempty(r));
            }
            if (!go) break;
            // the item's rows: two 32-column chunks through the staging buffer
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const uint32_t col = 64u * hc + 32u * c;
                if (col >= p.nt || uint32_t(m0) + q * 32u >= p.n || uint32_t(n0) + col >= p.k_out) continue;
                // the previous store from this buffer has read it
                if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                __syncwarp();
                uint8_t* row = gobuf + lane * 128u;
#pragma unroll
                for (uint32_t j = 0; j < 8; ++j)
                    *reinterpret_cast<float4*>(row + ((j ^ (lane & 7u)) * 16u)) =
                        make_float4(acc[32 * c + 4 * j], acc[32 * c + 4 * j + 1], acc[32 * c + 4 * j + 2],
                                    acc[32 * c + 4 * j + 3]);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) tma_store_2d(&tm_out, n0 + int(col), m0 + int(q * 32), obuf);
            }
        }
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
    }
}

// W (k_in x k_out, row-major) to K-major W^T (k_out x kp, kp = k_in rounded
// up to 4, zeros past k_in); in 3xTF32 also the split hi = rna(w), lo =
// rna(w - hi) of every value.
__global__ void transpose_w_kernel(const float* __restrict__ w, uint32_t k_in, uint32_t k_out, uint32_t kp,
                                   float* __restrict__ wt, float* __restrict__ wt_lo) {
    const size_t total = size_t(k_out) * kp;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const uint32_t j = uint32_t(i / kp), kk = uint32_t(i % kp);
        const float x = kk < k_in ? w[size_t(kk) * k_out + j] : 0.f;
        if (wt_lo) {
            const float h = tf32_hi(x);
            wt[i] = h;
            wt_lo[i] = tf32_hi(x - h);
        } else {
            wt[i] = tf32_hi(x);
        }
    }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (the library links the runtime statically and not libcuda).
int encode_tiled(EncodeTiledFn* out) {
    static std::mutex mu;
    static EncodeTiledFn fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000,
                                                               cudaEnableDefault, &q);
        if (e != cudaSuccess || !ptr || q != cudaDriverEntryPointSuccess)
            ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
        fn = reinterpret_cast<EncodeTiledFn>(ptr);
    }
    *out = fn;
    return ACCSPMM_SUCCESS;
}

// Tensor map of a row-major fp32 matrix of `rows` x `cols` (cols % 4 == 0,
// 16-byte aligned base) read in boxes of 32 columns x box_rows rows with
// 128-byte swizzle; reads past either edge return zeros.
int fp32_kmajor_map(EncodeTiledFn enc, CUtensorMap* tm, const float* base, uint64_t rows, uint64_t cols,
                    uint32_t box_rows) {
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 4};
    const cuuint32_t box[2] = {32u, box_rows};
    const cuuint32_t es[2] = {1, 1};
    const CUresult cr = enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, es,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) ACC_FAIL(ACCSPMM_ERROR_CUDA, "cuTensorMapEncodeTiled failed (%d)", int(cr));
    return ACCSPMM_SUCCESS;
}

int launch_gemm_ws(const CUtensorMap& th, const CUtensorMap& tw, const CUtensorMap& tout, WsParams p,
                   cudaStream_t s) {
    constexpr size_t kMaxDyn = 226 * 1024;
    const size_t fixed = 4 * 2 * kStageOut + 1024;  // store staging + alignment slack
    p.stage_bytes = kATileBytes + p.nt * 128u;
    uint32_t st = uint32_t((kMaxDyn - fixed) / p.stage_bytes);
    p.stages = st > 8 ? 8 : st;
    if (p.stages < 2) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "shared memory too small for two stages");
    size_t smem = size_t(p.stages) * p.stage_bytes + fixed;
    // one CTA per SM: more than half of the SM's 228 KB
    if (smem < 115 * 1024) smem = 115 * 1024;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(dense_gemm_tf32_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(kMaxDyn)));
        attr_set |= 1u << dev;
    }
    const uint32_t grid = std::min<uint32_t>(p.items, uint32_t(sm_count()));
    dense_gemm_tf32_ws_kernel<<<grid, kWsThreads, smem, s>>>(th, tw, tout, p);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

int launch_gemm_3xtf32_ws(const CUtensorMap& th, const CUtensorMap& tw, const CUtensorMap& twl,
                          const CUtensorMap& tout, WsParams p, cudaStream_t s) {
    constexpr size_t kMaxDyn = 226 * 1024;
    const size_t fixed = 8 * kStageOut + 1024;  // store staging + alignment slack
    p.stage_bytes = 2 * kATileBytes + 2 * p.nt * 128u;
    uint32_t st = uint32_t((kMaxDyn - fixed) / p.stage_bytes);
    p.stages = st > 4 ? 4 : st;
    if (p.stages < 2) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "shared memory too small for two stages");
    size_t smem = size_t(p.stages) * p.stage_bytes + fixed;
    if (smem < 115 * 1024) smem = 115 * 1024;  // one CTA per SM (it takes all 512 TMEM columns)
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(dense_gemm_3xtf32_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(kMaxDyn)));
        attr_set |= 1u << dev;
    }
    const uint32_t grid = std::min<uint32_t>(p.items, uint32_t(sm_count()));
    dense_gemm_3xtf32_ws_kernel<<<grid, kX3Threads, smem, s>>>(th, tw, twl, tout, p);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

}  // namespace

int dense_gemm_status_take(unsigned int* v) {
    ACC_CUDA(cudaMemcpyFromSymbol(v, g_gemm_status, sizeof *v));
    if (*v) {
        const unsigned int z = 0;
        ACC_CUDA(cudaMemcpyToSymbol(g_gemm_status, &z, sizeof z));
    }
    return ACCSPMM_SUCCESS;
}

int dense_gemm_impl(const float* H, uint32_t n, uint32_t k_in, const float* W, uint32_t k_out, float* XW,
                    int precision, cudaStream_t s) {
    if (k_in == 0 || k_out == 0 || k_out % 4)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "k_in > 0 and k_out a positive multiple of 4 required");
    if (precision != ACCSPMM_PREC_TF32 && precision != ACCSPMM_PREC_3XTF32)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    if (n == 0) return ACCSPMM_SUCCESS;  // nothing to read or write
    if (!H || !W || !XW) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "H, W and XW must be device pointers");
    if (reinterpret_cast<uintptr_t>(XW) & 15u) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "XW must be 16-byte aligned");
    const bool split = precision == ACCSPMM_PREC_3XTF32;
    cudaMemPool_t pool = nullptr;
    int r = library_pool(&pool);
    if (r) return r;
    EncodeTiledFn enc = nullptr;
    if ((r = encode_tiled(&enc))) return r;
    const uint32_t kp = (k_in + 3) & ~3u;
    // H as the tensor map needs it: 16-byte aligned rows of kp floats
    const float* h = H;
    float* hp = nullptr;
    float* wt = nullptr;
    auto give_back = [&]() {
        if (hp) cudaFreeAsync(hp, s);
        if (wt) cudaFreeAsync(wt, s);
    };
    if (kp != k_in || (reinterpret_cast<uintptr_t>(H) & 15u)) {
        const size_t bytes = size_t(n) * kp * 4;
        cudaError_t ce = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&hp), bytes, pool, s);
        if (ce != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_ALLOC, "pool allocation failed: %s", cudaGetErrorString(ce));
        ce = cudaMemsetAsync(hp, 0, bytes, s);
        if (ce == cudaSuccess)
            ce = cudaMemcpy2DAsync(hp, size_t(kp) * 4, H, size_t(k_in) * 4, size_t(k_in) * 4, n,
                                   cudaMemcpyDeviceToDevice, s);
        if (ce != cudaSuccess) {
            give_back();
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "copy of H failed: %s", cudaGetErrorString(ce));
        }
        h = hp;
    }
    // W^T, K-major (and its low parts in 3xTF32), rounded to TF32
    const size_t wn = size_t(k_out) * kp;
    cudaError_t ce = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&wt), wn * 4 * (split ? 2 : 1), pool, s);
    if (ce != cudaSuccess) {
        give_back();
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "pool allocation failed: %s", cudaGetErrorString(ce));
    }
    float* wt_lo = split ? wt + wn : nullptr;
    {
        const unsigned blocks = unsigned(std::min<size_t>((wn + 255) / 256, 4096));
        transpose_w_kernel<<<blocks, 256, 0, s>>>(W, k_in, k_out, kp, wt, wt_lo);
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) {
            give_back();
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "transpose launch failed: %s", cudaGetErrorString(le));
        }
    }
    // TF32: up to 256 output columns per work item, two alternating TMEM
    // accumulators; 3xTF32: up to 128, the four 128-column regions of two
    // k-blocks in flight (main and correction products each)
    WsParams w{};
    w.n = n;
    w.k_out = k_out;
    w.kblocks = (kp + kBK - 1) / kBK;
    w.nt = std::min<uint32_t>(split ? 128 : 256, (k_out + 15) & ~15u);
    w.n_tiles = (k_out + w.nt - 1) / w.nt;
    w.items = ((n + kBM - 1) / kBM) * w.n_tiles;  // below 2^32: n < 2^32, n_tiles <= 2^24 / 16
    w.acc_stride = 32;
    while (w.acc_stride < w.nt) w.acc_stride <<= 1;
    w.tmem_cols = split ? 512 : 2 * w.acc_stride;
    // XW written by tensor-map stores of 32 x 32 boxes (rows past n and
    // columns past k_out are not written)
    CUtensorMap th, tw, twl, tout;
    r = fp32_kmajor_map(enc, &th, h, n, kp, kBM);
    if (!r) r = fp32_kmajor_map(enc, &tw, wt, k_out, kp, w.nt);
    if (!r) r = fp32_kmajor_map(enc, &twl, split ? wt_lo : wt, k_out, kp, w.nt);
    if (!r) r = fp32_kmajor_map(enc, &tout, XW, n, k_out, 32);
    if (!r) r = split ? launch_gemm_3xtf32_ws(th, tw, twl, tout, w, s) : launch_gemm_ws(th, tw, tout, w, s);
    give_back();
    return r;
}

}  // namespace accspmm
