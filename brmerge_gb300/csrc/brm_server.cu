// brm_server.cu -- a request loop for many independent SpGEMM requests.
//
// Callers submit C = A * B requests (device CSR, Precise) from any thread and
// wait for them by ticket.  A submit only queues the request.  An admission
// thread takes every newly queued request at once, counts their products
// with one kernel on a high-priority stream (no per-request synchronisation,
// no shared context), turns them into upper-bound bytes, rejects those whose
// bound alone exceeds the memory cap and passes the others on.  Worker
// threads, each with its own context and non-blocking stream, take whatever
// is admitted (same value type, in arrival order, bounds within kSizeRatio of
// the oldest one's), reserve the summed bounds under the cap, and run them as
// one batch (brm_batch_precise: one stacked-operand pipeline).  Express
// workers take only small requests (bound up to express_bytes) and run them
// on the device's highest-priority streams, so small batches are scheduled
// ahead of the pending blocks of large ones.  A result stays in the batch's
// device arrays until the caller releases it; the batch's memory goes back
// when its last result is released.
//
// No counterpart in the reference (a library call per product).
#include <algorithm>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "brm_common.cuh"
#include "brm_kernels.h"
#include "brmerge.h"

namespace {

constexpr long long kSizeRatio = 16;  // largest bound ratio within one batch
constexpr int kAdmitThreads = 256;
constexpr int kAdmitChunk = kAdmitThreads * 8;  // A entries a block counts

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

// One request of an admission round: its A columns and B row pointers.
struct AdmitItem {
    const int *acol;
    const int *brpt;
    int nnz_a;
    int K;
};

// Products of every request of a round (compute_flop, spgemm.h:31-56):
// blockIdx.y is the request, blockIdx.x a chunk of its A entries.  out[2i]
// collects the products, out[2i+1] a flag for a column or a B row pointer
// that is not valid CSR.
__global__ void __launch_bounds__(kAdmitThreads) k_admit_count(const AdmitItem *items,
                                                              unsigned long long *out)
{
    const AdmitItem it = items[blockIdx.y];
    const long long j0 = (long long)blockIdx.x * kAdmitChunk;
    if (j0 >= it.nnz_a)
        return;
    const int j1 = (int)(j0 + kAdmitChunk < it.nnz_a ? j0 + kAdmitChunk : it.nnz_a);
    unsigned long long f = 0;
    bool bad = false;
    for (int j = (int)j0 + threadIdx.x; j < j1; j += kAdmitThreads) {
        const int c = it.acol[j];
        if ((unsigned)c < (unsigned)it.K) {
            const int b0 = it.brpt[c], b1 = it.brpt[c + 1];
            if (b0 < 0 || b1 < b0)
                bad = true;
            else
                f += (unsigned long long)(b1 - b0);
        } else {
            bad = true;
        }
    }
    __shared__ unsigned long long s_f[kAdmitThreads / 32];
    __shared__ int s_bad;
    if (threadIdx.x == 0)
        s_bad = 0;
    f = brm::warp_sum(f);
    if ((threadIdx.x & 31) == 0)
        s_f[threadIdx.x >> 5] = f;
    __syncthreads();
    if (bad)
        s_bad = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kAdmitThreads / 32; w++)
            t += s_f[w];
        atomicAdd(&out[2 * blockIdx.y], t);
        if (s_bad)
            atomicOr(&out[2 * blockIdx.y + 1], 1ull);
    }
}

// SM partitions (green contexts): the driver's entry points, looked up at
// run time so that the library needs no link-time driver dependency.
struct GreenApi {
    CUresult (*dev_get)(CUdevice *, int) = nullptr;
    CUresult (*get_res)(CUdevice, CUdevResource *, CUdevResourceType) = nullptr;
    CUresult (*split)(CUdevResource *, unsigned *, const CUdevResource *, CUdevResource *,
                      unsigned, unsigned) = nullptr;
    CUresult (*gen_desc)(CUdevResourceDesc *, CUdevResource *, unsigned) = nullptr;
    CUresult (*create)(CUgreenCtx *, CUdevResourceDesc, CUdevice, unsigned) = nullptr;
    CUresult (*destroy)(CUgreenCtx) = nullptr;
    CUresult (*to_ctx)(CUcontext *, CUgreenCtx) = nullptr;
    CUresult (*set_current)(CUcontext) = nullptr;
    CUresult (*get_current)(CUcontext *) = nullptr;

    template <typename F>
    static bool sym(const char *name, F &f)
    {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion(name, &p, 13000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p) {
            (void)cudaGetLastError();
            return false;
        }
        f = reinterpret_cast<F>(p);
        return true;
    }
    bool load()
    {
        return sym("cuDeviceGet", dev_get) && sym("cuDeviceGetDevResource", get_res) &&
               sym("cuDevSmResourceSplitByCount", split) &&
               sym("cuDevResourceGenerateDesc", gen_desc) && sym("cuGreenCtxCreate", create) &&
               sym("cuGreenCtxDestroy", destroy) && sym("cuCtxFromGreenCtx", to_ctx) &&
               sym("cuCtxSetCurrent", set_current) && sym("cuCtxGetCurrent", get_current);
    }
};

// One SM partition: a green context and its context handle.
struct Partition {
    CUgreenCtx green = nullptr;
    CUcontext ctx = nullptr;
    int sms = 0;
};

}  // namespace

struct brm_server_s {
    int device = 0;
    long long cap = 0;
    int max_batch = 0;
    long long express_bytes = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_admit;
    std::deque<Request *> pending;  // submitted, bound not yet known
    std::deque<Request *> queue;    // admitted to the work queue
    std::unordered_map<long long, Request *> all;
    long long next_ticket = 1;
    long long reserved = 0;  // bytes of admitted, unreleased requests
    bool stop = false;
    std::vector<std::thread> workers;
    std::vector<brm_context> ctxs;
    std::vector<cudaStream_t> streams;
    std::vector<char> express;  // per worker: takes only small requests
    std::thread admitter;
    cudaStream_t admit_stream = nullptr;
    // SM partitions: the express workers and the admission run on the SM set
    // res[0], the other workers on res[1].  A green context may be current
    // in one thread at a time, so every thread has one of its own (gctx[w]
    // for worker w, gctx_admit for the admission thread).
    GreenApi api;
    CUdevice cu_dev = 0;
    CUdevResource res[2] = {};
    int part_sms[2] = {0, 0};
    bool partitioned = false;
    std::vector<Partition> gctx;
    Partition gctx_admit;

    bool make_partitions(int express_sms);
    int new_green(int set, Partition *out);
    void drop_green(Partition &p)
    {
        if (p.green)
            api.destroy(p.green);
        p = Partition{};
    }
    // Makes the calling thread run on its own green context (or the device's
    // primary context when the SMs are not partitioned).
    void enter(const Partition &p)
    {
        if (partitioned && p.ctx)
            api.set_current(p.ctx);
        else
            cudaSetDevice(device);
    }

    void work(int w);
    void admit();
    void finish(Request *r, int status);
};

// Marks a request done without running it (rejected at admission); mu held.
void brm_server_s::finish(Request *r, int status)
{
    r->status = status;
    r->t_start = r->t_done = now_s();
    r->done = true;
}

// Splits the device's SMs into a partition of at least express_sms SMs (for
// the express workers and the admission) and the rest (for the other
// workers), one green context each.  False (nothing changed) when the driver
// or the device cannot.
bool brm_server_s::make_partitions(int express_sms)
{
    if (!api.load())
        return false;
    CUdevResource all{};
    unsigned ng = 1;
    if (api.dev_get(&cu_dev, device) != CUDA_SUCCESS ||
        api.get_res(cu_dev, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS ||
        api.split(&res[0], &ng, &all, &res[1], 0, (unsigned)express_sms) != CUDA_SUCCESS ||
        ng < 1 || res[0].sm.smCount == 0 || res[1].sm.smCount == 0)
        return false;
    part_sms[0] = (int)res[0].sm.smCount;
    part_sms[1] = (int)res[1].sm.smCount;
    partitioned = true;
    return true;
}

// A green context over SM set `set` (0: express, 1: the rest).
int brm_server_s::new_green(int set, Partition *out)
{
    *out = Partition{};
    CUdevResourceDesc desc;
    if (api.gen_desc(&desc, &res[set], 1) != CUDA_SUCCESS ||
        api.create(&out->green, desc, cu_dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS ||
        api.to_ctx(&out->ctx, out->green) != CUDA_SUCCESS) {
        drop_green(*out);
        return BRM_ERR_CUDA;
    }
    out->sms = part_sms[set];
    return BRM_SUCCESS;
}

void brm_server_s::admit()
{
    enter(gctx_admit);
    AdmitItem *d_items = nullptr, *h_items = nullptr;
    unsigned long long *d_out = nullptr, *h_out = nullptr;
    int cap_items = 0;
    for (;;) {
        std::vector<Request *> round;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_admit.wait(lk, [&] { return stop || !pending.empty(); });
            if (pending.empty() && stop)
                break;
            while (!pending.empty() && round.size() < 65535) {
                round.push_back(pending.front());
                pending.pop_front();
            }
        }
        const int n = (int)round.size();
        int st = BRM_SUCCESS;
        if (n > cap_items) {
            cudaFree(d_items);
            cudaFreeHost(h_items);
            cudaFree(d_out);
            cudaFreeHost(h_out);
            d_items = h_items = nullptr;
            d_out = h_out = nullptr;
            cap_items = std::max(n, 256);
            if (cudaMalloc(&d_items, sizeof(AdmitItem) * cap_items) != cudaSuccess ||
                cudaMallocHost(&h_items, sizeof(AdmitItem) * cap_items) != cudaSuccess ||
                cudaMalloc(&d_out, 16 * (size_t)cap_items) != cudaSuccess ||
                cudaMallocHost(&h_out, 16 * (size_t)cap_items) != cudaSuccess) {
                (void)cudaGetLastError();
                cap_items = 0;
                st = BRM_ERR_ALLOC;
            }
        }
        int max_nnz = 0;
        if (st == BRM_SUCCESS) {
            for (int i = 0; i < n; i++) {
                const Request *r = round[(size_t)i];
                h_items[i] = AdmitItem{r->A.col, r->B.rpt, r->A.nnz, r->B.M};
                max_nnz = std::max(max_nnz, r->A.nnz);
            }
            const dim3 grid((unsigned)std::max(1, (max_nnz + kAdmitChunk - 1) / kAdmitChunk),
                            (unsigned)n);
            cudaError_t e = cudaMemcpyAsync(d_items, h_items, sizeof(AdmitItem) * (size_t)n,
                                            cudaMemcpyHostToDevice, admit_stream);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(d_out, 0, 16 * (size_t)n, admit_stream);
            if (e == cudaSuccess) {
                k_admit_count<<<grid, kAdmitThreads, 0, admit_stream>>>(d_items, d_out);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(h_out, d_out, 16 * (size_t)n, cudaMemcpyDeviceToHost,
                                    admit_stream);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(admit_stream);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                st = BRM_ERR_CUDA;
            }
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            for (int i = 0; i < n; i++) {
                Request *r = round[(size_t)i];
                if (st != BRM_SUCCESS) {
                    finish(r, st);
                    continue;
                }
                if (h_out[2 * i + 1]) {
                    finish(r, BRM_ERR_INVALID_CSR);
                    continue;
                }
                const long long prod = (long long)h_out[2 * i];
                const long long vb = r->dtype == BRM_F64 ? 8 : 4;
                // the Upper bound of C plus the operands' stacked copies
                r->bound = brm::upper_bound_bytes(r->dtype, r->A.M, prod) +
                           2 * ((long long)r->A.nnz * (4 + vb) + (long long)r->B.nnz * (4 + vb) +
                                4ll * ((long long)r->A.M + r->B.M + 2));
                if (r->bound > cap)
                    finish(r, BRM_ERR_CAPACITY);
                else
                    queue.push_back(r);
            }
        }
        cv_work.notify_all();
        cv_done.notify_all();
    }
    cudaFree(d_items);
    cudaFreeHost(h_items);
    cudaFree(d_out);
    cudaFreeHost(h_out);
}

void brm_server_s::work(int w)
{
    const bool small_only = express[(size_t)w] != 0;
    enter(gctx[(size_t)w]);
    brm_context ctx = ctxs[(size_t)w];
    for (;;) {
        std::vector<Request *> batch;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (stop && queue.empty() && pending.empty())
                    return;
                // first fit in arrival order: the head's value type, while
                // the admitted bytes stay under the cap (the head is always
                // admitted when nothing else is in flight); requests whose
                // bounds differ from the head's by more than kSizeRatio wait
                // for a batch of their own size, so a small request does not
                // wait for a large one's batch.  An express worker's head is
                // the oldest small request.
                auto head = queue.begin();
                if (small_only)
                    while (head != queue.end() && (*head)->bound > express_bytes)
                        ++head;
                if (head != queue.end()) {
                    const brm_dtype dt = (*head)->dtype;
                    const long long hb = std::max((*head)->bound, 1LL);
                    for (auto it = head; it != queue.end() && (int)batch.size() < max_batch;) {
                        Request *r = *it;
                        const long long rb = std::max(r->bound, 1LL);
                        if (r->dtype != dt || rb > hb * kSizeRatio || rb * kSizeRatio < hb ||
                            (small_only && r->bound > express_bytes)) {
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
    const int nx = cfg ? (cfg->express_workers < 0 ? 0 : std::min(cfg->express_workers, 16)) : 1;
    srv->express_bytes = (cfg && cfg->express_bytes > 0) ? cfg->express_bytes : (64ll << 20);
    const int xsms = cfg ? cfg->express_sms : 0;
    cudaGetDevice(&srv->device);
    int lo = 0, hi = 0;  // stream priorities: hi is the most urgent (numerically lowest)
    int st = cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess ? BRM_SUCCESS : BRM_ERR_CUDA;
    // SM partitions for the express workers (when the driver offers them)
    CUcontext caller = nullptr;
    if (st == BRM_SUCCESS && nx > 0 && xsms >= 0 && srv->make_partitions(xsms > 0 ? xsms : 16))
        srv->api.get_current(&caller);
    srv->gctx.assign((size_t)(nw + nx), Partition{});
    auto leave = [&] {
        if (srv->partitioned)
            srv->api.set_current(caller);
    };
    if (st == BRM_SUCCESS && srv->partitioned)
        st = srv->new_green(0, &srv->gctx_admit);
    if (st == BRM_SUCCESS) {
        srv->enter(srv->gctx_admit);
        if (cudaStreamCreateWithPriority(&srv->admit_stream, cudaStreamNonBlocking, hi) !=
            cudaSuccess)
            st = BRM_ERR_CUDA;
    }
    for (int w = 0; w < nw + nx && st == BRM_SUCCESS; w++) {
        const bool xw = w >= nw;
        if (srv->partitioned) {
            st = srv->new_green(xw ? 0 : 1, &srv->gctx[(size_t)w]);
            if (st != BRM_SUCCESS)
                break;
        }
        // the worker's context, streams and events belong to its own
        // context (green when partitioned)
        srv->enter(srv->gctx[(size_t)w]);
        brm_context c = nullptr;
        cudaStream_t s = nullptr;
        st = brm_create(&c);
        if (st != BRM_SUCCESS)
            break;
        if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, xw ? hi : lo) != cudaSuccess) {
            (void)cudaGetLastError();
            brm_destroy(c);
            st = BRM_ERR_CUDA;
            break;
        }
        brm_set_stream(c, s);
        if (xw)
            st = brm::set_context_priority(c, hi);
        if (st == BRM_SUCCESS && srv->partitioned)
            st = brm::set_context_sms(c, srv->gctx[(size_t)w].sms);
        srv->ctxs.push_back(c);
        srv->streams.push_back(s);
        srv->express.push_back(xw ? 1 : 0);
    }
    if (st != BRM_SUCCESS) {
        (void)cudaGetLastError();
        for (size_t w = 0; w < srv->ctxs.size(); w++) {
            srv->enter(srv->gctx[w]);
            brm_destroy(srv->ctxs[w]);
            cudaStreamDestroy(srv->streams[w]);
        }
        srv->enter(srv->gctx_admit);
        if (srv->admit_stream)
            cudaStreamDestroy(srv->admit_stream);
        leave();
        for (Partition &p : srv->gctx)
            srv->drop_green(p);
        srv->drop_green(srv->gctx_admit);
        delete srv;
        return st;
    }
    leave();
    srv->admitter = std::thread([srv] { srv->admit(); });
    for (int w = 0; w < nw + nx; w++)
        srv->workers.emplace_back([srv, w] { srv->work(w); });
    *out = srv;
    return BRM_SUCCESS;
}

int brm_server_sms(brm_server srv, int *express_sms, int *other_sms)
{
    if (!srv || !express_sms || !other_sms)
        return BRM_ERR_INVALID_VALUE;
    *express_sms = srv->partitioned ? srv->part_sms[0] : 0;
    *other_sms = srv->partitioned ? srv->part_sms[1] : 0;
    return BRM_SUCCESS;
}

int brm_server_submit(brm_server srv, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                      long long *ticket)
{
    if (!srv || !A || !B || !ticket || (dtype != BRM_F64 && dtype != BRM_F32))
        return BRM_ERR_INVALID_VALUE;
    if (A->N != B->M || A->M < 0 || B->M < 0 || B->N < 0 || A->nnz < 0 || B->nnz < 0 ||
        !A->rpt || !B->rpt || (A->nnz > 0 && !A->col))
        return BRM_ERR_INVALID_VALUE;
    auto *r = new (std::nothrow) Request();
    if (!r)
        return BRM_ERR_ALLOC;
    r->t_submit = now_s();
    r->dtype = dtype;
    r->A = *A;
    r->B = *B;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) {
            delete r;
            return BRM_ERR_INVALID_VALUE;
        }
        r->ticket = srv->next_ticket++;
        srv->all[r->ticket] = r;
        srv->pending.push_back(r);
        *ticket = r->ticket;
    }
    srv->cv_admit.notify_one();
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
    srv->cv_admit.notify_all();
    srv->admitter.join();  // every pending request is admitted or rejected
    srv->cv_work.notify_all();
    for (auto &t : srv->workers)
        t.join();
    for (auto &kv : srv->all)
        delete kv.second;
    srv->all.clear();
    CUcontext caller = nullptr;
    if (srv->partitioned)
        srv->api.get_current(&caller);
    for (size_t w = 0; w < srv->ctxs.size(); w++) {
        srv->enter(srv->gctx[w]);
        brm_destroy(srv->ctxs[w]);
        cudaStreamDestroy(srv->streams[w]);
    }
    srv->enter(srv->gctx_admit);
    cudaStreamDestroy(srv->admit_stream);
    if (srv->partitioned) {
        srv->api.set_current(caller);
        for (Partition &p : srv->gctx)
            srv->drop_green(p);
        srv->drop_green(srv->gctx_admit);
    }
    delete srv;
    return BRM_SUCCESS;
}

}  // extern "C"
