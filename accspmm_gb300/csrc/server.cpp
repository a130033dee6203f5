// server.cpp -- a continuous-batching SpMM request server.
//
// METCF matrices stay resident on the device.  Callers submit requests
// (matrix, host B, host C, K, precision, chain length) from any thread.  A
// worker thread admits pending requests in arrival order while the device
// memory they need (B, C and a chain temporary) fits in the HBM budget and a
// launch slot (stream) is free, groups them into one batch, and enqueues on
// that slot's stream: the host->device copies of every B, one batched
// persistent launch (two for two-layer chains A (A B)), the device->host
// copies of every C, stream-ordered frees, and a host callback that marks
// the requests done and releases their budget.  Requests that arrive while
// earlier batches are on the GPU are admitted as soon as memory and a slot
// free up, so their work overlaps on the device.  Each request is computed
// by the same per-item arithmetic whatever else is in its batch, so its
// result does not depend on the mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "accspmm.h"
#include "common.hpp"
#include "spmm_batch.hpp"

namespace accspmm {
namespace {

using Clock = std::chrono::steady_clock;

double now_s() {
    return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t id = 0;
    uint32_t graph = 0, K = 0, chain = 1;
    int precision = ACCSPMM_PREC_TF32;
    const float* B_host = nullptr;
    float* C_host = nullptr;
    size_t bytes_B = 0, bytes_C = 0, bytes_T = 0;
    double t_submit = 0, t_done = 0;
    int status = ACCSPMM_SUCCESS;
    bool done = false, cancelled = false;
    float* dB = nullptr;
    float* dC = nullptr;
    float* dT = nullptr;
    size_t bytes() const { return bytes_B + bytes_C + bytes_T; }
};

}  // namespace

struct ServerImpl;

struct ServedBatch {
    ServerImpl* srv = nullptr;
    int slot = -1;
    std::vector<std::shared_ptr<Request>> reqs;
    BatchDesc* d_desc = nullptr;  // [2n] descriptors (two passes) + work counter
    uint32_t* d_counter = nullptr;
};

struct ServerImpl {
    int device = 0;
    std::vector<accspmm_metcf_t> graphs;
    accspmm_server_config_t cfg{};
    std::vector<cudaStream_t> streams;
    std::vector<bool> slot_busy;
    std::vector<BatchDesc*> staging;  // pinned, 2 max_batch descriptors per slot

    std::mutex mu;
    std::condition_variable cv;  // worker wake-up and completion notices
    std::deque<std::shared_ptr<Request>> pending;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> all;
    uint64_t next_id = 1;
    size_t used = 0, peak = 0;
    uint64_t submitted = 0, completed = 0, rejected = 0, cancelled = 0, launches = 0;
    uint64_t batched_requests = 0;
    double first_submit = 0, last_done = 0;
    std::vector<double> lat_ms;
    int fatal = ACCSPMM_SUCCESS;
    bool stop = false;
    std::thread worker;

    void run();
    int issue(std::vector<std::shared_ptr<Request>>& take, int slot, uint32_t* passes);
    static void CUDART_CB on_done(void* p);
};

namespace {

// Descriptors of one pass go through the slot's pinned staging area (free
// again once the slot's previous batch has completed), then one launch.
int enqueue_pass(const std::vector<BatchInput>& in, int precision, BatchDesc* staging,
                 BatchDesc* d_desc, uint32_t* d_counter, cudaStream_t s) {
    uint32_t total = 0, max_wb = 1, max_k = 4;
    for (auto& x : in) max_k = std::max(max_k, x.K);
    const int fs = batch_fs_for(max_k);
    std::vector<BatchDesc> desc;
    int st = make_batch_descs(in.data(), uint32_t(in.size()), fs, precision, &desc, &total, &max_wb);
    if (st) return st;
    if (total == 0) return ACCSPMM_SUCCESS;
    std::copy(desc.begin(), desc.end(), staging);
    cudaError_t e = cudaMemcpyAsync(d_desc, staging, sizeof(BatchDesc) * desc.size(),
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_CUDA, "descriptor copy: %s", cudaGetErrorString(e));
    return launch_batch(d_desc, uint32_t(desc.size()), total, max_wb, d_counter, fs, precision, s);
}

}  // namespace

void CUDART_CB ServerImpl::on_done(void* p) {
    // runs on a CUDA callback thread: no CUDA calls here
    std::unique_ptr<ServedBatch> b(static_cast<ServedBatch*>(p));
    ServerImpl* s = b->srv;
    const double t = now_s();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        for (auto& r : b->reqs) {
            r->t_done = t;
            r->done = true;
            s->used -= r->bytes();
            s->completed++;
            s->lat_ms.push_back((t - r->t_submit) * 1e3);
            s->last_done = t;
        }
        s->slot_busy[b->slot] = false;
    }
    s->cv.notify_all();
}

int ServerImpl::issue(std::vector<std::shared_ptr<Request>>& take, int slot, uint32_t* passes) {
    cudaStream_t st = streams[slot];
    std::unique_ptr<ServedBatch> b(new ServedBatch());
    b->srv = this;
    b->slot = slot;
    b->reqs = take;
    const size_t n = take.size();
    *passes = 0;
    // On a failure part of the batch may already be enqueued (copies into
    // C_host among them): wait for the slot's stream, so that nothing still
    // writes a caller's buffer once its request reports the failure, then
    // free the buffers whose stream-ordered frees were not enqueued.
    auto bail = [&](int code) {
        cudaStreamSynchronize(st);
        for (auto& r : take) {
            for (float** q : {&r->dB, &r->dC, &r->dT})
                if (*q) {
                    cudaFree(*q);
                    *q = nullptr;
                }
        }
        if (b->d_desc) cudaFree(b->d_desc);
        b->d_desc = nullptr;
        return code;
    };
#define SERVER_FAIL(code, ...)             \
    do {                                   \
        ::accspmm::set_error(__VA_ARGS__); \
        return bail(code);                 \
    } while (0)
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&b->d_desc), sizeof(BatchDesc) * 2 * n + 16, st);
    if (e != cudaSuccess) {
        b->d_desc = nullptr;
        SERVER_FAIL(ACCSPMM_ERROR_ALLOC, "descriptor allocation: %s", cudaGetErrorString(e));
    }
    b->d_counter = reinterpret_cast<uint32_t*>(b->d_desc + 2 * n);
    std::vector<BatchInput> in(n);
    for (size_t i = 0; i < n; ++i) {
        Request& r = *take[i];
        const accspmm_metcf_t& m = graphs[r.graph];
        e = cudaMallocAsync(reinterpret_cast<void**>(&r.dB), r.bytes_B, st);
        if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&r.dC), r.bytes_C, st);
        if (e == cudaSuccess && r.bytes_T) e = cudaMallocAsync(reinterpret_cast<void**>(&r.dT), r.bytes_T, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(r.dB, r.B_host, r.bytes_B, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) SERVER_FAIL(ACCSPMM_ERROR_CUDA, "request buffers: %s", cudaGetErrorString(e));
        // the first layer of a chain writes the temporary, else C
        in[i] = BatchInput{m.row_window_offset, m.tc_offset, m.tc_local_bit, m.sparse_a2b, m.data,
                           r.dB, r.chain == 2 ? r.dT : r.dC, m.num_windows, m.num_windows,
                           m.num_tiles, m.cols, r.K};
    }
    BatchDesc* stg = staging[slot];
    int rc = enqueue_pass(in, take[0]->precision, stg, b->d_desc, b->d_counter, st);
    if (rc) return bail(rc);
    *passes = 1;
    // second layer of two-layer chains: C = A (A B), the temporary is its B
    std::vector<BatchInput> in2;
    for (size_t i = 0; i < n; ++i)
        if (take[i]->chain == 2) {
            BatchInput x = in[i];
            x.B = take[i]->dT;
            x.C = take[i]->dC;
            in2.push_back(x);
        }
    if (!in2.empty()) {
        rc = enqueue_pass(in2, take[0]->precision, stg + n, b->d_desc + n, b->d_counter, st);
        if (rc) return bail(rc);
        *passes = 2;
    }
    for (auto& r : take) {
        e = cudaMemcpyAsync(r->C_host, r->dC, r->bytes_C, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) SERVER_FAIL(ACCSPMM_ERROR_CUDA, "result copy: %s", cudaGetErrorString(e));
    }
    for (auto& r : take) {
        for (float** q : {&r->dB, &r->dC, &r->dT})
            if (*q) {
                cudaFreeAsync(*q, st);
                *q = nullptr;
            }
    }
    cudaFreeAsync(b->d_desc, st);
    b->d_desc = nullptr;
    e = cudaLaunchHostFunc(st, &ServerImpl::on_done, b.get());
    if (e != cudaSuccess) SERVER_FAIL(ACCSPMM_ERROR_CUDA, "completion callback: %s", cudaGetErrorString(e));
#undef SERVER_FAIL
    b.release();  // owned by the callback now
    return ACCSPMM_SUCCESS;
}

void ServerImpl::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(mu);
    for (;;) {
        cv.wait(lock, [&] {
            if (stop && pending.empty()) return true;
            if (pending.empty()) return false;
            for (bool b : slot_busy)
                if (!b) return true;
            return false;
        });
        if (stop && pending.empty()) return;
        int slot = -1;
        for (size_t i = 0; i < slot_busy.size(); ++i)
            if (!slot_busy[i]) {
                slot = int(i);
                break;
            }
        if (slot < 0) continue;
        // admit in arrival order: same precision as the oldest request, while
        // the HBM budget and the batch size allow
        std::vector<std::shared_ptr<Request>> take;
        const int prec = pending.front()->precision;
        size_t add = 0;
        for (auto it = pending.begin(); it != pending.end() && take.size() < cfg.max_batch;) {
            Request& r = **it;
            if (r.precision != prec) {
                ++it;
                continue;
            }
            if (used + add + r.bytes() > cfg.hbm_budget_bytes) break;
            add += r.bytes();
            take.push_back(*it);
            it = pending.erase(it);
        }
        if (take.empty()) {
            // the oldest request does not fit yet: wait for completions
            cv.wait(lock);
            continue;
        }
        used += add;
        peak = std::max(peak, used);
        slot_busy[slot] = true;
        batched_requests += take.size();
        lock.unlock();
        uint32_t passes = 0;
        int rc = issue(take, slot, &passes);
        lock.lock();
        launches += passes;
        if (rc) {
            // a failed enqueue ends the server; the requests carry the status
            fatal = rc;
            for (auto& r : take) {
                r->status = rc;
                r->done = true;
                used -= r->bytes();
            }
            slot_busy[slot] = false;
            cv.notify_all();
        }
    }
}

}  // namespace accspmm

using accspmm::ServerImpl;
using accspmm::Request;

struct accspmm_server {
    ServerImpl impl;
};

extern "C" {

int accspmm_server_create(const accspmm_metcf_t* graphs, uint32_t n_graphs,
                          const accspmm_server_config_t* cfg, accspmm_server_t** out) {
    accspmm::clear_error();
    if (!out || (n_graphs && !graphs) || !cfg) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    *out = nullptr;
    for (uint32_t i = 0; i < n_graphs; ++i)
        if (graphs[i].space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "graph %u is not on the device", i);
    auto* s = new accspmm_server();
    ServerImpl& im = s->impl;
    cudaGetDevice(&im.device);
    im.graphs.assign(graphs, graphs + n_graphs);
    im.cfg = *cfg;
    if (im.cfg.max_batch == 0) im.cfg.max_batch = 64;
    if (im.cfg.streams == 0) im.cfg.streams = 4;
    im.streams.resize(im.cfg.streams);
    im.slot_busy.assign(im.cfg.streams, false);
    im.staging.assign(im.cfg.streams, nullptr);
    for (uint32_t i = 0; i < im.cfg.streams; ++i) {
        if (cudaStreamCreateWithFlags(&im.streams[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaMallocHost(reinterpret_cast<void**>(&im.staging[i]),
                           sizeof(accspmm::BatchDesc) * 2 * im.cfg.max_batch) != cudaSuccess) {
            delete s;
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "stream or staging allocation failed");
        }
    }
    im.worker = std::thread([&im] { im.run(); });
    *out = s;
    return ACCSPMM_SUCCESS;
}

int accspmm_server_submit(accspmm_server_t* s, uint32_t graph, const float* B_host, float* C_host,
                          uint32_t K, int32_t precision, uint32_t chain, uint64_t* request_id) {
    accspmm::clear_error();
    if (!s || !B_host || !C_host || !request_id) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    ServerImpl& im = s->impl;
    if (graph >= im.graphs.size()) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "graph %u out of range", graph);
    if (K == 0 || K % 4) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K=%u must be a positive multiple of 4", K);
    if (precision != ACCSPMM_PREC_TF32 && precision != ACCSPMM_PREC_3XTF32)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    if (chain != 1 && chain != 2) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "chain must be 1 or 2");
    const accspmm_metcf_t& m = im.graphs[graph];
    if (chain == 2 && m.rows != m.cols) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "a two-layer chain needs a square matrix");
    auto r = std::make_shared<Request>();
    r->graph = graph;
    r->K = K;
    r->chain = chain;
    r->precision = precision;
    r->B_host = B_host;
    r->C_host = C_host;
    r->bytes_B = size_t(m.cols) * K * 4;
    r->bytes_C = size_t(m.num_windows) * 8 * K * 4;
    r->bytes_T = chain == 2 ? r->bytes_C : 0;
    r->t_submit = accspmm::now_s();
    {
        std::lock_guard<std::mutex> lock(im.mu);
        if (im.stop) ACC_FAIL(ACCSPMM_ERROR_CANCELLED, "server is shutting down");
        if (im.fatal) ACC_FAIL(im.fatal, "server stopped after an earlier failure");
        if (r->bytes() > im.cfg.hbm_budget_bytes) {
            im.rejected++;
            ACC_FAIL(ACCSPMM_ERROR_ADMISSION, "request needs %zu bytes, budget is %zu", r->bytes(),
                     im.cfg.hbm_budget_bytes);
        }
        r->id = im.next_id++;
        if (im.submitted == 0) im.first_submit = r->t_submit;
        im.submitted++;
        im.all[r->id] = r;
        im.pending.push_back(r);
        *request_id = r->id;
    }
    im.cv.notify_all();
    return ACCSPMM_SUCCESS;
}

int accspmm_server_wait(accspmm_server_t* s, uint64_t request_id, int32_t timeout_ms) {
    accspmm::clear_error();
    if (!s) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null server");
    ServerImpl& im = s->impl;
    std::unique_lock<std::mutex> lock(im.mu);
    auto it = im.all.find(request_id);
    if (it == im.all.end()) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown request %llu", (unsigned long long)request_id);
    std::shared_ptr<Request> r = it->second;
    auto done = [&] { return r->done; };
    if (timeout_ms < 0) im.cv.wait(lock, done);
    else if (!im.cv.wait_for(lock, std::chrono::milliseconds(timeout_ms), done))
        ACC_FAIL(ACCSPMM_ERROR_TIMEOUT, "request %llu not done after %d ms", (unsigned long long)request_id, timeout_ms);
    im.all.erase(request_id);
    if (r->status) ACC_FAIL(r->status, "request %llu %s", (unsigned long long)request_id,
                            r->cancelled ? "was cancelled" : "failed");
    return ACCSPMM_SUCCESS;
}

int accspmm_server_cancel(accspmm_server_t* s, uint64_t request_id) {
    accspmm::clear_error();
    if (!s) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null server");
    ServerImpl& im = s->impl;
    std::lock_guard<std::mutex> lock(im.mu);
    for (auto it = im.pending.begin(); it != im.pending.end(); ++it)
        if ((*it)->id == request_id) {
            (*it)->cancelled = true;
            (*it)->status = ACCSPMM_ERROR_CANCELLED;
            (*it)->done = true;
            im.cancelled++;
            im.pending.erase(it);
            im.cv.notify_all();
            return ACCSPMM_SUCCESS;
        }
    ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "request %llu is not pending", (unsigned long long)request_id);
}

int accspmm_server_stats(accspmm_server_t* s, accspmm_server_stats_t* out) {
    accspmm::clear_error();
    if (!s || !out) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    ServerImpl& im = s->impl;
    std::lock_guard<std::mutex> lock(im.mu);
    std::memset(out, 0, sizeof *out);
    out->submitted = im.submitted;
    out->completed = im.completed;
    out->rejected = im.rejected;
    out->cancelled = im.cancelled;
    out->launches = im.launches;
    out->peak_bytes = im.peak;
    out->mean_batch = im.launches ? double(im.batched_requests) / double(im.launches) : 0.0;
    if (!im.lat_ms.empty()) {
        std::vector<double> v = im.lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) { return v[std::min(v.size() - 1, size_t(q * double(v.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_ms = sum / double(v.size());
        const double span = im.last_done - im.first_submit;
        out->throughput_rps = span > 0 ? double(im.completed) / span : 0.0;
    }
    return im.fatal;
}

int accspmm_server_reset_stats(accspmm_server_t* s) {
    accspmm::clear_error();
    if (!s) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null server");
    ServerImpl& im = s->impl;
    std::lock_guard<std::mutex> lock(im.mu);
    im.lat_ms.clear();
    im.submitted = im.completed = im.rejected = im.cancelled = im.launches = im.batched_requests = 0;
    im.first_submit = im.last_done = 0;
    im.peak = im.used;
    return ACCSPMM_SUCCESS;
}

void accspmm_server_destroy(accspmm_server_t* s) {
    if (!s) return;
    ServerImpl& im = s->impl;
    {
        std::lock_guard<std::mutex> lock(im.mu);
        im.stop = true;
    }
    im.cv.notify_all();
    if (im.worker.joinable()) im.worker.join();
    for (auto& st : im.streams) {
        if (!st) continue;
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (auto* p : im.staging) cudaFreeHost(p);
    delete s;
}

}  // extern "C"
