// brm_server.cu -- a request loop for many independent SpGEMM requests.
//
// Callers submit C = A * B requests (device CSR, Precise) from any thread and
// wait for them by ticket.  Worker threads, each with its own context and
// non-blocking stream, take whatever is queued (same value type, in arrival
// order), admit requests while the summed upper-bound bytes of everything
// admitted and not yet released stay under the memory cap, and run them as
// one batch (brm_batch_precise: one stacked-operand pipeline).  Requests that
// arrive while batches are on the GPU wait for the next free worker, so the
// batches of different workers overlap on the device.  A result stays in
// the batch's device arrays until the caller releases it; the batch's memory
// goes back when its last result is released.
//
// No counterpart in the reference (a library call per product).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "brmerge.h"

namespace {

constexpr long long kSizeRatio = 16;  // largest bound ratio within one batch

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Device arrays of one finished batch, shared by its requests; freed on the
// server's device by whichever thread releases the last of them.
struct BatchMem {
    brm_batch b{};
    int device = 0;
    ~BatchMem()
    {
        int cur = 0;
        cudaGetDevice(&cur);
        if (cur != device)
            cudaSetDevice(device);
        brm_batch_free(nullptr, &b);
        if (cur != device)
            cudaSetDevice(cur);
    }
};

struct Request {
    long long ticket = 0;
    brm_dtype dtype = BRM_F64;
    brm_csr A{}, B{};
    long long bound = 0;   // admission bytes
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = BRM_SUCCESS;
    bool done = false;
    bool admitted = false;
    std::shared_ptr<BatchMem> mem;
    int idx = 0;
    int batch_size = 0;
};

}  // namespace

struct brm_server_s {
    int device = 0;
    long long cap = 0;
    int max_batch = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::unordered_map<long long, Request *> all;
    long long next_ticket = 1;
    long long reserved = 0;  // bytes of admitted, unreleased requests
    bool stop = false;
    std::vector<std::thread> workers;
    std::vector<brm_context> ctxs;
    std::vector<cudaStream_t> streams;
    brm_context admit_ctx = nullptr;  // upper-bound estimates at submit
    std::mutex admit_mu;

    void work(int w);
};

void brm_server_s::work(int w)
{
    cudaSetDevice(device);
    brm_context ctx = ctxs[(size_t)w];
    for (;;) {
        std::vector<Request *> batch;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (stop && queue.empty())
                    return;
                if (!queue.empty()) {
                    // first fit in arrival order: the head's value type, while
                    // the admitted bytes stay under the cap (the head is always
                    // admitted when nothing else is in flight)
                    // requests whose bounds differ from the head's by more
                    // than kSizeRatio wait for a batch of their own size, so a
                    // small request does not wait for a large one's batch
                    const brm_dtype dt = queue.front()->dtype;
                    const long long hb = std::max(queue.front()->bound, 1LL);
                    for (auto it = queue.begin();
                         it != queue.end() && (int)batch.size() < max_batch;) {
                        Request *r = *it;
                        const long long rb = std::max(r->bound, 1LL);
                        if (r->dtype != dt || rb > hb * kSizeRatio || rb * kSizeRatio < hb) {
                            ++it;
                            continue;
                        }
                        if (reserved + r->bound > cap && !(reserved == 0 && batch.empty()))
                            break;
                        reserved += r->bound;
                        r->admitted = true;
                        batch.push_back(r);
                        it = queue.erase(it);
                    }
                    if (!batch.empty())
                        break;
                }
                cv_work.wait(lk);
            }
        }
        const double t0 = now_s();
        const int n = (int)batch.size();
        std::vector<brm_csr> As((size_t)n), Bs((size_t)n);
        for (int i = 0; i < n; i++) {
            As[(size_t)i] = batch[(size_t)i]->A;
            Bs[(size_t)i] = batch[(size_t)i]->B;
        }
        auto mem = std::make_shared<BatchMem>();
        mem->device = device;
        const int st = brm_batch_precise(ctx, batch[0]->dtype, n, As.data(), Bs.data(), &mem->b);
        const double t1 = now_s();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (int i = 0; i < n; i++) {
                Request *r = batch[(size_t)i];
                r->t_start = t0;
                r->t_done = t1;
                r->status = st;
                r->idx = i;
                r->batch_size = n;
                if (st == BRM_SUCCESS)
                    r->mem = mem;
                r->done = true;
            }
        }
        cv_done.notify_all();
    }
}

extern "C" {

int brm_server_create(const brm_server_config *cfg, brm_server *out)
{
    if (!out)
        return BRM_ERR_INVALID_VALUE;
    *out = nullptr;
    brm_server srv = new (std::nothrow) brm_server_s();
    if (!srv)
        return BRM_ERR_ALLOC;
    srv->cap = (cfg && cfg->mem_cap_bytes > 0) ? cfg->mem_cap_bytes : (60ll << 30);
    srv->max_batch = (cfg && cfg->max_batch > 0) ? cfg->max_batch : 4096;
    const int nw = (cfg && cfg->workers > 0) ? std::min(cfg->workers, 16) : 2;
    cudaGetDevice(&srv->device);
    int st = brm_create(&srv->admit_ctx);
    for (int w = 0; w < nw && st == BRM_SUCCESS; w++) {
        brm_context c = nullptr;
        cudaStream_t s = nullptr;
        st = brm_create(&c);
        if (st != BRM_SUCCESS)
            break;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            (void)cudaGetLastError();
            brm_destroy(c);
            st = BRM_ERR_CUDA;
            break;
        }
        brm_set_stream(c, s);
        srv->ctxs.push_back(c);
        srv->streams.push_back(s);
    }
    if (st != BRM_SUCCESS) {
        for (brm_context c : srv->ctxs)
            brm_destroy(c);
        for (cudaStream_t s : srv->streams)
            cudaStreamDestroy(s);
        if (srv->admit_ctx)
            brm_destroy(srv->admit_ctx);
        delete srv;
        return st;
    }
    for (int w = 0; w < nw; w++)
        srv->workers.emplace_back([srv, w] { srv->work(w); });
    *out = srv;
    return BRM_SUCCESS;
}

int brm_server_submit(brm_server srv, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                      long long *ticket)
{
    if (!srv || !A || !B || !ticket || (dtype != BRM_F64 && dtype != BRM_F32))
        return BRM_ERR_INVALID_VALUE;
    if (A->N != B->M || A->M < 0 || B->N < 0)
        return BRM_ERR_INVALID_VALUE;
    auto *r = new (std::nothrow) Request();
    if (!r)
        return BRM_ERR_ALLOC;
    r->t_submit = now_s();
    r->dtype = dtype;
    r->A = *A;
    r->B = *B;
    {
        // admission estimate: the Upper bound of C plus the operands' copies
        std::lock_guard<std::mutex> g(srv->admit_mu);
        long long prod = 0, bytes = 0;
        const int st = brm_upper_bound(srv->admit_ctx, dtype, A, B, &prod, &bytes);
        if (st != BRM_SUCCESS) {
            delete r;
            return st;
        }
        const long long vb = dtype == BRM_F64 ? 8 : 4;
        r->bound = bytes + 2 * ((long long)A->nnz * (4 + vb) + (long long)B->nnz * (4 + vb) +
                                4ll * ((long long)A->M + B->M + 2));
    }
    if (r->bound > srv->cap) {
        delete r;
        return BRM_ERR_CAPACITY;
    }
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) {
            delete r;
            return BRM_ERR_INVALID_VALUE;
        }
        r->ticket = srv->next_ticket++;
        srv->all[r->ticket] = r;
        srv->queue.push_back(r);
        *ticket = r->ticket;
    }
    srv->cv_work.notify_one();
    return BRM_SUCCESS;
}

int brm_server_wait(brm_server srv, long long ticket, double timeout_s, brm_server_result *out)
{
    if (!srv || !out)
        return BRM_ERR_INVALID_VALUE;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->all.find(ticket);
    if (it == srv->all.end())
        return BRM_ERR_INVALID_VALUE;
    Request *r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_s < 0)
        srv->cv_done.wait(lk, ready);
    else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
        return BRM_ERR_TIMEOUT;
    std::memset(out, 0, sizeof(*out));
    out->status = r->status;
    out->M = r->A.M;
    out->N = r->B.N;
    out->queued_s = r->t_start - r->t_submit;
    out->latency_s = r->t_done - r->t_submit;
    out->batch_size = r->batch_size;
    if (r->status == BRM_SUCCESS && r->mem) {
        const brm_batch &b = r->mem->b;
        const long long r0 = b.row_off[r->idx], n0 = b.nnz_off[r->idx];
        const size_t vb = r->dtype == BRM_F64 ? 8 : 4;
        out->nnz = (int)(b.nnz_off[r->idx + 1] - n0);
        out->rpt = b.rpt_local + r0 + r->idx;
        out->col = b.ccol + n0;
        out->val = (const char *)b.cval + vb * (size_t)n0;
    }
    return r->status;
}

int brm_server_release(brm_server srv, long long ticket)
{
    if (!srv)
        return BRM_ERR_INVALID_VALUE;
    Request *r = nullptr;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        auto it = srv->all.find(ticket);
        if (it == srv->all.end() || !it->second->done)
            return BRM_ERR_INVALID_VALUE;
        r = it->second;
        srv->all.erase(it);
        if (r->admitted)
            srv->reserved -= r->bound;
    }
    delete r;  // the batch's arrays go with its last request
    srv->cv_work.notify_all();
    return BRM_SUCCESS;
}

int brm_server_destroy(brm_server srv)
{
    if (!srv)
        return BRM_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (auto &t : srv->workers)
        t.join();
    for (auto &kv : srv->all)
        delete kv.second;
    srv->all.clear();
    for (brm_context c : srv->ctxs)
        brm_destroy(c);
    for (cudaStream_t s : srv->streams)
        cudaStreamDestroy(s);
    brm_destroy(srv->admit_ctx);
    delete srv;
    return BRM_SUCCESS;
}

}  // extern "C"
