// brm_hostpool.cu -- page-locked host blocks for the results of the host
// drop-ins (brm_precise, brm_upper and their float forms).
//
// The reference hands back C = A*B in arrays the call allocates and the
// caller frees (BRMerge-SpGEMM/inc/spgemm.h:575-578, :414-418).  The GPU
// form returns its result from device memory, and a device-to-host copy into
// freshly malloc'ed (pageable) memory runs at a fraction of the host link's
// bandwidth and pays a page fault per page.  The result arrays therefore come
// from page-locked blocks that brm_free hands back to this cache, so a
// caller that multiplies repeatedly copies straight into pinned memory.
//
// Blocks are cached by capacity (multiples of 2 MiB).  A request takes the
// smallest cached block that is at least as large and at most twice as
// large; freed blocks beyond BRM_HOST_CACHE_MB (default 16384) of cached
// capacity go back to the driver.  When page-locking fails the block comes
// from malloc instead and brm_free releases it with free.
#include <cstdlib>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "brm_hostpool.h"

namespace brm {
namespace {

constexpr size_t kGranule = size_t(2) << 20;

struct HostPool {
    std::mutex mu;
    std::multimap<size_t, void *> idle;       // capacity -> cached block
    std::unordered_map<void *, size_t> lent;  // block handed out -> capacity
    size_t idle_bytes = 0;
    size_t limit = 0;

    HostPool()
    {
        size_t mb = 16384;
        if (const char *s = std::getenv("BRM_HOST_CACHE_MB")) {
            char *end = nullptr;
            const unsigned long long v = std::strtoull(s, &end, 10);
            if (end != s)
                mb = (size_t)v;
        }
        limit = mb << 20;
    }
};

// Never destroyed: blocks may still be lent out while static destructors
// run, and the CUDA runtime may already be gone then.
HostPool &pool()
{
    static HostPool *p = new HostPool();
    return *p;
}

}  // namespace

void *host_alloc(size_t bytes)
{
    const size_t need = ((bytes ? bytes : 1) + kGranule - 1) / kGranule * kGranule;
    HostPool &P = pool();
    {
        std::lock_guard<std::mutex> g(P.mu);
        auto it = P.idle.lower_bound(need);
        if (it != P.idle.end() && it->first <= 2 * need) {
            void *p = it->second;
            const size_t cap = it->first;
            P.idle.erase(it);
            P.idle_bytes -= cap;
            P.lent.emplace(p, cap);
            return p;
        }
    }
    void *p = nullptr;
    if (cudaHostAlloc(&p, need, cudaHostAllocDefault) != cudaSuccess) {
        (void)cudaGetLastError();
        return std::malloc(bytes ? bytes : 1);
    }
    std::lock_guard<std::mutex> g(P.mu);
    P.lent.emplace(p, need);
    return p;
}

bool host_release(void *p)
{
    HostPool &P = pool();
    size_t cap = 0;
    {
        std::lock_guard<std::mutex> g(P.mu);
        auto it = P.lent.find(p);
        if (it == P.lent.end())
            return false;
        cap = it->second;
        P.lent.erase(it);
        if (P.idle_bytes + cap <= P.limit) {
            P.idle.emplace(cap, p);
            P.idle_bytes += cap;
            return true;
        }
    }
    cudaFreeHost(p);
    (void)cudaGetLastError();
    return true;
}

void host_trim()
{
    HostPool &P = pool();
    std::vector<void *> blocks;
    {
        std::lock_guard<std::mutex> g(P.mu);
        for (auto &kv : P.idle)
            blocks.push_back(kv.second);
        P.idle.clear();
        P.idle_bytes = 0;
    }
    for (void *p : blocks)
        cudaFreeHost(p);
    (void)cudaGetLastError();
}

}  // namespace brm
