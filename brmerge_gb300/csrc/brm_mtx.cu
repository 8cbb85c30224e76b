// brm_mtx.cu -- MatrixMarket coordinate reader into device CSR.
//
// Replaces the reference's CSR::construct (BRMerge-SpGEMM/src/CSR.cpp:259-479),
// which reads the body with one stream extraction per token, expands
// symmetric formats and sorts (row, column) keys on one core.  Here the
// header (banner, comments, size line) is parsed on the host, the body is
// streamed into device memory through page-locked staging blocks, and the
// device does the rest:
//   k_txt_count   token starts per 16 KB block of text
//   (scan)        first token index of every block
//   k_txt_parse   every token: field = index mod F, entry = index div F;
//                 integers checked against M and N, reals converted with
//                 correct rounding (brm_numparse.h); the few reals the device
//                 cannot decide are converted exactly on the host
//   k_mtx_keys    64-bit (row, column) keys, mirrors of symmetric entries
//   k_rs_hist / k_rs_scatter   stable LSD radix sort of the keys (8 bits a
//                 pass, only the bits the sizes need)
//   k_mtx_csr     columns, values, row pointers; repeated keys are errors
//                 (the reference rejects them as "not in ascending order",
//                 CSR.cpp:454-466)
#include <fcntl.h>
#include <locale.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "brm_common.cuh"
#include "brm_hostpool.h"
#include "brm_kernels.h"
#include "brm_numparse.h"
#include "brmerge.h"

namespace brm {
namespace {

__device__ const uint64_t d_pow5[kPow5Rows][2] = {BRM_POW5_ROWS};

constexpr int kTxtThreads = 256;
constexpr int kTxtBytes = 64;                        // text bytes per thread
constexpr int kTxtBlock = kTxtThreads * kTxtBytes;   // 16 KB per block
constexpr int kHalo = 256;                           // bytes staged past a block
constexpr int kPad = 64;                             // whitespace after the body
constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;       // items per sort block
constexpr int kSlotBytes = 64;                       // deferred-token slot
constexpr size_t kStageBytes = 32u << 20;            // staging block size
constexpr int kStageSlots = 4;

enum MtxErr : int {
    kMtxBadToken = 1,  // a token that is not an integer / a real
    kMtxRow = 2,       // row index outside [1, M] (or a mirror outside)
    kMtxCol = 4,       // column index outside [1, N]
    kMtxDup = 8,       // repeated (row, column)
};

struct MtxCnt {
    int err;
    int pad;
    unsigned long long slow;     // reals deferred to the host
    unsigned long long offdiag;  // off-diagonal entries (symmetric formats)
    unsigned long long mirror;   // mirrors written so far
};

struct SlowTok {
    long long pos;    // byte offset in the body
    long long entry;  // entry index
};

__device__ __forceinline__ void mtx_fail(MtxCnt *c, int code) { atomicOr(&c->err, code); }

// 64-bit mask of the token starts among the 64 bytes at b0 (a start is a
// non-space byte after a space or at the start of the body).
__device__ __forceinline__ unsigned long long start_mask(const unsigned char *txt, long long b0)
{
    const uint4 *p = (const uint4 *)(txt + b0);
    unsigned prev = b0 > 0 ? txt[b0 - 1] : ' ';
    unsigned long long m = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const uint4 u = p[q];
        const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const unsigned c = (w[k >> 2] >> (8 * (k & 3))) & 0xffu;
            if (!tok_space(c) && tok_space(prev))
                m |= 1ull << (q * 16 + k);
            prev = c;
        }
    }
    return m;
}

__global__ void __launch_bounds__(kTxtThreads) k_txt_count(const unsigned char *txt, int *blk)
{
    __shared__ int ws[kTxtThreads / 32 + 1];
    const long long b0 = (long long)blockIdx.x * kTxtBlock + (long long)threadIdx.x * kTxtBytes;
    const int c = __popcll(start_mask(txt, b0));
    const int s = block_sum<kTxtThreads>(c, ws);
    if (threadIdx.x == 0)
        blk[blockIdx.x] = s;
}

// Bytes of the text as staged by k_txt_parse: the block and its halo from
// shared memory, anything further from global memory.
struct StagedText {
    const unsigned char *st;  // shared copy of [blk0, blk0 + in_smem)
    const unsigned char *txt;
    long long at0;            // offset of byte 0 of the token from blk0
    int in_smem;
    __device__ unsigned operator()(int i) const
    {
        const long long o = at0 + i;
        return o < in_smem ? st[o] : txt[o];
    }
};

// Every token of the block: F fields per entry (2 pattern, 3 real/integer,
// 4 complex); tokens from ntok on are ignored.
template <int F>
__global__ void __launch_bounds__(kTxtThreads)
    k_txt_parse(const unsigned char *txt, long long alloc, const long long *blk_base,
                long long ntok, int M, int N, int *I, int *J, double *V, MtxCnt *cnt,
                SlowTok *slow)
{
    __shared__ __align__(16) unsigned char st[kTxtBlock + kHalo];
    __shared__ long long ws[kTxtThreads / 32 + 1];
    const long long blk0 = (long long)blockIdx.x * kTxtBlock;
    const long long b0 = blk0 + (long long)threadIdx.x * kTxtBytes;
    // stage the block and a halo (alloc - blk0 is a multiple of 16)
    const int in_smem = (int)min((long long)(kTxtBlock + kHalo), alloc - blk0);
    {
        const uint4 *src = (const uint4 *)(txt + blk0);
        uint4 *dst = (uint4 *)st;
        for (int i = threadIdx.x; i < (in_smem >> 4); i += kTxtThreads)
            dst[i] = src[i];
    }
    unsigned long long m = start_mask(txt, b0);
    long long tot;
    long long g = blk_base[blockIdx.x] +
                  block_excl_scan<kTxtThreads, long long>(__popcll(m), ws, &tot);
    // (block_excl_scan ends with a barrier: the staged text is visible)
    const unsigned char *gtxt = txt + blk0;
    while (m && g < ntok) {
        const int j = __ffsll((long long)m) - 1;
        m &= m - 1;
        const long long pos = b0 + j;
        const StagedText at{st, gtxt, pos - blk0, in_smem};
        int len = 0;  // the body is followed by whitespace, so this ends
        while (!tok_space(at(len)))
            len++;
        const long long e = g / F;
        const int f = (int)(g - e * F);
        g++;
        if (f < 2) {
            long long v;
            if (parse_int_at(at, len, &v) != kTokOk) {
                mtx_fail(cnt, kMtxBadToken);
                continue;
            }
            const long long x = v - 1;
            if (f == 0) {
                if (x < 0 || x >= M)
                    mtx_fail(cnt, kMtxRow);
                else
                    I[e] = (int)x;
            } else {
                if (x < 0 || x >= N)
                    mtx_fail(cnt, kMtxCol);
                else
                    J[e] = (int)x;
            }
            continue;
        }
        double v = 0.0;
        const int r = parse_real_at(at, len, f == 2 ? d_pow5 : nullptr, &v);
        if (r == kTokBad) {
            mtx_fail(cnt, kMtxBadToken);
        } else if (f == 2) {
            if (r == kTokOk) {
                V[e] = v;
            } else {
                // exact conversion on the host
                const unsigned long long k = atomicAdd(&cnt->slow, 1ull);
                slow[k] = SlowTok{pos, e};
            }
        }
    }
}

// Deferred tokens: their first kSlotBytes - 1 bytes and full length.
__global__ void k_slow_gather(const unsigned char *txt, const SlowTok *slow, long long n,
                              unsigned char *slots, int *lens)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned char *p = txt + slow[i].pos;
        int len = 0;
        while (!tok_space(p[len])) {
            if (len < kSlotBytes - 1)
                slots[i * kSlotBytes + len] = p[len];
            len++;
        }
        lens[i] = len;
    }
}

__global__ void k_slow_scatter(const SlowTok *slow, const double *vals, long long n, double *V)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        if (slow[i].entry >= 0)
            V[slow[i].entry] = vals[i];
}

__global__ void k_offdiag(const int *I, const int *J, long long nnz, MtxCnt *cnt)
{
    __shared__ unsigned long long ws[8 + 1];
    unsigned long long c = 0;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz;
         e += (long long)gridDim.x * blockDim.x)
        c += I[e] != J[e];
    c = block_sum<256>(c, ws);
    if (threadIdx.x == 0 && c)
        atomicAdd(&cnt->offdiag, c);
}

// (row << cb) | col keys; mirrors of off-diagonal entries after the nnz
// entries (their order does not matter: the keys are sorted and unique).
template <bool SYM, bool SKEW, bool PATTERN>
__global__ void k_mtx_keys(const int *I, const int *J, const double *V, long long nnz, int cb,
                           int M, int N, unsigned long long *key, double *val, MtxCnt *cnt)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz;
         e += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r = (unsigned)I[e], c = (unsigned)J[e];
        const double v = PATTERN ? 1.0 : V[e];
        key[e] = (r << cb) | c;
        val[e] = v;
        if (SYM && r != c) {
            if (c >= (unsigned long long)M || r >= (unsigned long long)N) {
                mtx_fail(cnt, kMtxRow);  // the mirror falls outside the matrix
                continue;
            }
            const long long k = nnz + (long long)atomicAdd(&cnt->mirror, 1ull);
            key[k] = (c << cb) | r;
            val[k] = SKEW ? -v : v;
        }
    }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const unsigned long long *key, int n,
                                                        int shift, int nblk, int *hist)
{
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kRsTile;
#pragma unroll 4
    for (int it = 0; it < kRsItems; it++) {
        const long long i = base + it * kRsThreads + threadIdx.x;
        if (i < n)
            atomicAdd(&h[(key[i] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one radix pass: warp w of a block owns items
// [base + 512 w, base + 512 w + 512) and walks them 32 at a time in order;
// an item's rank among the block's items of its digit is the count from
// earlier warps plus earlier items of its own warp.
__global__ void __launch_bounds__(kRsThreads)
    k_rs_scatter(const unsigned long long *kin, const double *vin, int n, int shift, int nblk,
                 const long long *off, unsigned long long *kout, double *vout)
{
    constexpr int NW = kRsThreads / 32;
    __shared__ int wc[NW][256];
    __shared__ long long boff[256];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    boff[tid] = off[(long long)tid * nblk + blockIdx.x];
#pragma unroll
    for (int q = 0; q < NW; q++)
        wc[q][tid] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kRsTile + (long long)w * (kRsItems * 32);
    unsigned long long k[kRsItems];
    double v[kRsItems];
    int r[kRsItems];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int it = 0; it < kRsItems; it++) {
        const long long i = base + it * 32 + lane;
        const bool ok = i < n;
        k[it] = ok ? kin[i] : 0ull;
        v[it] = ok ? vin[i] : 0.0;
        const int d = ok ? (int)((k[it] >> shift) & 255) : 256 + lane;
        const unsigned peers = __match_any_sync(kFull, d);
        r[it] = ok ? wc[w][d] + __popc(peers & lt) : 0;
        __syncwarp();
        if (ok && (peers >> lane) == 1u)  // last lane of its group
            wc[w][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        int run = 0;
#pragma unroll
        for (int q = 0; q < NW; q++) {
            const int c = wc[q][tid];
            wc[q][tid] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kRsItems; it++) {
        const long long i = base + it * 32 + lane;
        if (i < n) {
            const int d = (int)((k[it] >> shift) & 255);
            const long long p = boff[d] + wc[w][d] + r[it];
            kout[p] = k[it];
            vout[p] = v[it];
        }
    }
}

template <typename T>
__global__ void k_mtx_csr(const unsigned long long *key, const double *val, int n, int cb, int M,
                          int *rpt, int *col, T *out, MtxCnt *cnt)
{
    const unsigned long long cmask = (1ull << cb) - 1ull;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long k = key[i];
        const int r = (int)(k >> cb);
        col[i] = (int)(k & cmask);
        out[i] = (T)val[i];
        int pr = -1;
        if (i > 0) {
            const unsigned long long kp = key[i - 1];
            if (kp == k)
                mtx_fail(cnt, kMtxDup);
            pr = (int)(kp >> cb);
        }
        for (int q = pr + 1; q <= r; q++)
            rpt[q] = (int)i;
        if (i == n - 1)
            for (int q = r + 1; q <= M; q++)
                rpt[q] = n;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// tokenize() of CSR.cpp:22-39: split on " \t\r\n"
std::vector<std::string> split_ws(const std::string &line)
{
    std::vector<std::string> t;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && std::strchr(" \t\r\n", line[i]) && line[i])
            i++;
        size_t j = i;
        while (j < line.size() && !(std::strchr(" \t\r\n", line[j]) && line[j]))
            j++;
        if (j > i)
            t.push_back(line.substr(i, j - i));
        i = j;
    }
    return t;
}

bool read_line(FILE *f, std::string &line)
{
    line.clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f)) != EOF) {
        any = true;
        if (c == '\n')
            return true;
        line.push_back((char)c);
    }
    return any;
}

bool host_int(const std::string &t, long long *v)
{
    return parse_int_tok((const unsigned char *)t.data(), (int)t.size(), v) == kTokOk;
}

struct Header {
    long long M = 0, N = 0, nnz = 0;
    int fields = 3;
    bool pattern = false, sym = false, skew = false;
    long long body_off = 0, body_len = 0;
};

// Banner, comments and size line (CSR.cpp:42-79, :265-288).
int read_header(const char *path, Header *h)
{
    FILE *f = std::fopen(path, "rb");
    if (!f)
        return BRM_ERR_IO;
    std::string line;
    int st = BRM_SUCCESS;
    do {
        if (!read_line(f, line)) {
            st = BRM_ERR_FORMAT;
            break;
        }
        std::vector<std::string> b = split_ws(line);
        if (b.size() != 5 || b[0] != "%%MatrixMarket" || b[1] != "matrix" ||
            b[2] != "coordinate") {
            st = BRM_ERR_FORMAT;
            break;
        }
        if (b[3] == "pattern") {
            h->fields = 2;
            h->pattern = true;
        } else if (b[3] == "real" || b[3] == "integer") {
            h->fields = 3;
        } else if (b[3] == "complex") {
            h->fields = 4;
        } else {
            st = BRM_ERR_FORMAT;
            break;
        }
        if (b[4] == "symmetric") {
            h->sym = true;
        } else if (b[4] == "skew-symmetric") {
            h->sym = h->skew = true;
        } else if (b[4] != "general") {
            st = BRM_ERR_FORMAT;
            break;
        }
        bool got = false;
        while (read_line(f, line)) {
            if (!line.empty() && line[0] == '%')
                continue;
            got = true;
            break;
        }
        if (!got) {
            st = BRM_ERR_FORMAT;
            break;
        }
        std::vector<std::string> s = split_ws(line);
        if (s.size() != 3 || !host_int(s[0], &h->M) || !host_int(s[1], &h->N) ||
            !host_int(s[2], &h->nnz) || h->M < 0 || h->N < 0 || h->nnz <= 0) {
            st = BRM_ERR_FORMAT;
            break;
        }
        h->body_off = std::ftell(f);
        if (h->body_off < 0 || std::fseek(f, 0, SEEK_END) != 0) {
            st = BRM_ERR_IO;
            break;
        }
        const long long end = std::ftell(f);
        h->body_len = end - h->body_off;
        if (h->body_len < 0)
            h->body_len = 0;
    } while (false);
    std::fclose(f);
    return st;
}

int bits_for(long long x)  // bits to hold values 0..x
{
    int b = 0;
    while (x > 0) {
        b++;
        x >>= 1;
    }
    return b;
}

int cuda_st(cudaError_t e)
{
    if (e == cudaSuccess)
        return BRM_SUCCESS;
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? BRM_ERR_ALLOC : BRM_ERR_CUDA;
}

#define MTX_CK(call)                    \
    do {                                \
        const int s_ = cuda_st(call);   \
        if (s_ != BRM_SUCCESS)          \
            return s_;                  \
    } while (0)

#define BRM_TRY_MTX(call)               \
    do {                                \
        const int s_ = (call);          \
        if (s_ != BRM_SUCCESS)          \
            return s_;                  \
    } while (0)

// Device temporaries of one read, released on every exit path.
struct Scratch {
    cudaStream_t s;
    std::vector<void *> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
    ~Scratch()
    {
        for (void *p : ptrs)
            cudaFreeAsync(p, s);
    }
    template <typename P>
    int alloc(P **p, size_t bytes)
    {
        void *q = nullptr;
        const int st = cuda_st(cudaMallocAsync(&q, bytes ? bytes : 16, s));
        if (st == BRM_SUCCESS)
            ptrs.push_back(q);
        *p = (P *)q;
        return st;
    }
};

// File body -> device: pread into page-locked staging blocks, each copied
// asynchronously while the next block is read.
int upload_body(const char *path, const Header &h, unsigned char *dtxt, cudaStream_t s)
{
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0)
        return BRM_ERR_IO;
    const size_t blk = (size_t)std::min<long long>(h.body_len, (long long)kStageBytes);
    void *stage[kStageSlots] = {};
    cudaEvent_t ev[kStageSlots] = {};
    int st = BRM_SUCCESS;
    for (int i = 0; i < kStageSlots && st == BRM_SUCCESS; i++) {
        stage[i] = host_alloc(blk);
        if (!stage[i])
            st = BRM_ERR_ALLOC;
        else
            st = cuda_st(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    }
    long long done = 0;
    for (int c = 0; st == BRM_SUCCESS && done < h.body_len; c++) {
        const int slot = c % kStageSlots;
        if (c >= kStageSlots) {
            st = cuda_st(cudaEventSynchronize(ev[slot]));
            if (st != BRM_SUCCESS)
                break;
        }
        const size_t want = (size_t)std::min<long long>((long long)blk, h.body_len - done);
        size_t got = 0;
        while (got < want) {
            const ssize_t r = ::pread(fd, (char *)stage[slot] + got, want - got,
                                      (off_t)(h.body_off + done + (long long)got));
            if (r <= 0) {
                st = BRM_ERR_IO;
                break;
            }
            got += (size_t)r;
        }
        if (st != BRM_SUCCESS)
            break;
        st = cuda_st(cudaMemcpyAsync(dtxt + done, stage[slot], want, cudaMemcpyHostToDevice, s));
        if (st == BRM_SUCCESS)
            st = cuda_st(cudaEventRecord(ev[slot], s));
        done += (long long)want;
    }
    const int st2 = cuda_st(cudaStreamSynchronize(s));
    if (st == BRM_SUCCESS)
        st = st2;
    for (int i = 0; i < kStageSlots; i++) {
        if (ev[i])
            cudaEventDestroy(ev[i]);
        if (stage[i] && !host_release(stage[i]))
            std::free(stage[i]);
    }
    ::close(fd);
    return st;
}

// Exact conversion of the deferred reals (strtod in the "C" locale, which
// rounds correctly), written back into V.
int convert_slow(const unsigned char *dtxt, long long nslow, const SlowTok *dslow, double *dV,
                 cudaStream_t s)
{
    Scratch sc(s);
    unsigned char *dslots;
    int *dlens;
    double *dvals;
    int st = sc.alloc(&dslots, (size_t)nslow * kSlotBytes);
    if (st == BRM_SUCCESS)
        st = sc.alloc(&dlens, (size_t)nslow * 4);
    if (st == BRM_SUCCESS)
        st = sc.alloc(&dvals, (size_t)nslow * 8);
    if (st != BRM_SUCCESS)
        return st;
    const int g = (int)std::min<long long>((nslow + 255) / 256, 4096);
    k_slow_gather<<<g, 256, 0, s>>>(dtxt, dslow, nslow, dslots, dlens);
    count_launch();
    std::vector<unsigned char> slots((size_t)nslow * kSlotBytes);
    std::vector<int> lens((size_t)nslow);
    std::vector<SlowTok> toks((size_t)nslow);
    MTX_CK(cudaMemcpyAsync(slots.data(), dslots, slots.size(), cudaMemcpyDeviceToHost, s));
    MTX_CK(cudaMemcpyAsync(lens.data(), dlens, lens.size() * 4, cudaMemcpyDeviceToHost, s));
    MTX_CK(cudaMemcpyAsync(toks.data(), dslow, toks.size() * sizeof(SlowTok),
                           cudaMemcpyDeviceToHost, s));
    MTX_CK(cudaStreamSynchronize(s));
    // tokens longer than a slot: copied one by one (rare)
    std::vector<std::string> longtok;
    std::vector<long long> longidx;
    for (long long i = 0; i < nslow; i++) {
        if (lens[(size_t)i] >= kSlotBytes) {
            std::string t((size_t)lens[(size_t)i], '\0');
            MTX_CK(cudaMemcpy(&t[0], dtxt + toks[(size_t)i].pos, t.size(),
                              cudaMemcpyDeviceToHost));
            longidx.push_back(i);
            longtok.push_back(std::move(t));
        }
    }
    std::vector<double> vals((size_t)nslow);
    locale_t cl = newlocale(LC_NUMERIC_MASK, "C", (locale_t)0);
    if (!cl)
        return BRM_ERR_ALLOC;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = nslow < 65536 ? 1u : std::min(16u, hw);
    std::vector<int> bad(nt, 0);
    auto convert = [&](const char *p, int len, double *out) {
        if (parse_real_tok((const unsigned char *)p, len, nullptr, out) == kTokBad)
            return false;  // (the device already checked; kept for long tokens)
        std::string t(p, (size_t)len);
        char *end = nullptr;
        const double v = strtod_l(t.c_str(), &end, cl);
        if (end != t.c_str() + len || std::isinf(v))
            return false;  // overflow: the reference's extraction fails here
        *out = v;
        return true;
    };
    for (size_t k = 0; k < longidx.size(); k++) {
        if (!convert(longtok[k].data(), (int)longtok[k].size(), &vals[(size_t)longidx[k]]))
            bad[0] = 1;
    }
    auto work = [&](unsigned t) {
        const long long per = (nslow + nt - 1) / nt;
        const long long i0 = (long long)t * per, i1 = std::min(nslow, i0 + per);
        for (long long i = i0; i < i1; i++) {
            const int len = lens[(size_t)i];
            if (len >= kSlotBytes)
                continue;
            if (!convert((const char *)&slots[(size_t)i * kSlotBytes], len, &vals[(size_t)i]))
                bad[t] = 1;
        }
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; t++)
            th.emplace_back(work, t);
        for (auto &x : th)
            x.join();
    }
    freelocale(cl);
    for (int b : bad)
        if (b)
            return BRM_ERR_FORMAT;
    MTX_CK(cudaMemcpyAsync(dvals, vals.data(), vals.size() * 8, cudaMemcpyHostToDevice, s));
    k_slow_scatter<<<g, 256, 0, s>>>(dslow, dvals, nslow, dV);
    count_launch();
    MTX_CK(cudaStreamSynchronize(s));  // vals (pageable) must outlive the copy
    return BRM_SUCCESS;
}

template <bool SYM, bool SKEW>
void launch_keys(bool pattern, const int *I, const int *J, const double *V, long long nnz, int cb,
                 int M, int N, unsigned long long *key, double *val, MtxCnt *cnt, int grid,
                 cudaStream_t s)
{
    if (pattern)
        k_mtx_keys<SYM, SKEW, true><<<grid, 256, 0, s>>>(I, J, V, nnz, cb, M, N, key, val, cnt);
    else
        k_mtx_keys<SYM, SKEW, false><<<grid, 256, 0, s>>>(I, J, V, nnz, cb, M, N, key, val, cnt);
    count_launch();
}

struct ReadOut {
    int M = 0, N = 0, nnz = 0;
    int *rpt = nullptr, *col = nullptr;
    void *val = nullptr;
};

// The whole read on `s`; on success the outputs are device allocations of
// the stream-ordered pool.
int read_device(const char *path, brm_dtype dtype, cudaStream_t s, int num_sms, ReadOut *out,
                brm_mtx_timing *tm)
{
    const double t0 = now_s();
    Header h;
    BRM_TRY_MTX(read_header(path, &h));
    const int F = h.fields;
    const long long nnz = h.nnz;
    const long long ntok = nnz * F;
    if (h.body_len <= 0)
        return BRM_ERR_FORMAT;
    const long long nb = h.body_len;
    const long long nblk = (nb + kTxtBlock - 1) / kTxtBlock;
    if (nblk > INT_MAX / 2)
        return BRM_ERR_CAPACITY;
    const long long alloc = nblk * kTxtBlock + kPad + kHalo;
    Scratch sc(s);
    unsigned char *dtxt;
    BRM_TRY_MTX(sc.alloc(&dtxt, (size_t)alloc));
    MTX_CK(cudaMemsetAsync(dtxt + nb, ' ', (size_t)(alloc - nb), s));
    BRM_TRY_MTX(upload_body(path, h, dtxt, s));
    const double t1 = now_s();

    // tokens
    int *blk;
    long long *base;
    void *stmp;
    MtxCnt *dcnt;
    int *I, *J;
    double *V = nullptr;
    SlowTok *slow = nullptr;
    BRM_TRY_MTX(sc.alloc(&blk, (size_t)nblk * 4));
    BRM_TRY_MTX(sc.alloc(&base, (size_t)(nblk + 1) * 8));
    BRM_TRY_MTX(sc.alloc(&stmp, scan_tmp_bytes((int)nblk)));
    BRM_TRY_MTX(sc.alloc(&dcnt, sizeof(MtxCnt)));
    BRM_TRY_MTX(sc.alloc(&I, (size_t)nnz * 4));
    BRM_TRY_MTX(sc.alloc(&J, (size_t)nnz * 4));
    if (!h.pattern) {
        BRM_TRY_MTX(sc.alloc(&V, (size_t)nnz * 8));
        BRM_TRY_MTX(sc.alloc(&slow, (size_t)nnz * sizeof(SlowTok)));
    }
    MTX_CK(cudaMemsetAsync(dcnt, 0, sizeof(MtxCnt), s));
    k_txt_count<<<(unsigned)nblk, kTxtThreads, 0, s>>>(dtxt, blk);
    count_launch();
    launch_scan_i64(blk, base, (int)nblk, stmp, s);
    const int M = (int)h.M, N = (int)h.N;
    if (F == 2)
        k_txt_parse<2><<<(unsigned)nblk, kTxtThreads, 0, s>>>(dtxt, alloc, base, ntok, M, N, I, J,
                                                               V, dcnt, slow);
    else if (F == 3)
        k_txt_parse<3><<<(unsigned)nblk, kTxtThreads, 0, s>>>(dtxt, alloc, base, ntok, M, N, I, J,
                                                               V, dcnt, slow);
    else
        k_txt_parse<4><<<(unsigned)nblk, kTxtThreads, 0, s>>>(dtxt, alloc, base, ntok, M, N, I, J,
                                                               V, dcnt, slow);
    count_launch();
    if (h.sym) {
        k_offdiag<<<num_sms * 4, 256, 0, s>>>(I, J, nnz, dcnt);
        count_launch();
    }
    MtxCnt hc;
    long long total_tok = 0;
    MTX_CK(cudaMemcpyAsync(&hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, s));
    MTX_CK(cudaMemcpyAsync(&total_tok, base + nblk, 8, cudaMemcpyDeviceToHost, s));
    MTX_CK(cudaStreamSynchronize(s));
    if (total_tok < ntok || hc.err)
        return BRM_ERR_FORMAT;
    if (hc.slow)
        BRM_TRY_MTX(convert_slow(dtxt, (long long)hc.slow, slow, V, s));
    const double t2 = now_s();

    // keys, sort, CSR
    const long long n2 = nnz + (h.sym ? (long long)hc.offdiag : 0);
    if (n2 > INT_MAX)
        return BRM_ERR_OVERFLOW;
    const int n = (int)n2;
    const int cb = bits_for((long long)N - 1);
    const int kbits = bits_for((long long)M - 1) + cb;
    unsigned long long *k0, *k1;
    double *v0, *v1;
    BRM_TRY_MTX(sc.alloc(&k0, (size_t)n * 8));
    BRM_TRY_MTX(sc.alloc(&v0, (size_t)n * 8));
    const int kgrid = (int)std::min<long long>((nnz + 255) / 256, (long long)num_sms * 16);
    if (!h.sym)
        launch_keys<false, false>(h.pattern, I, J, V, nnz, cb, M, N, k0, v0, dcnt, kgrid, s);
    else if (!h.skew)
        launch_keys<true, false>(h.pattern, I, J, V, nnz, cb, M, N, k0, v0, dcnt, kgrid, s);
    else
        launch_keys<true, true>(h.pattern, I, J, V, nnz, cb, M, N, k0, v0, dcnt, kgrid, s);
    const int npass = (kbits + 7) / 8;
    if (npass > 0) {
        const int rblk = (n + kRsTile - 1) / kRsTile;
        int *hist;
        long long *off;
        void *rtmp;
        BRM_TRY_MTX(sc.alloc(&k1, (size_t)n * 8));
        BRM_TRY_MTX(sc.alloc(&v1, (size_t)n * 8));
        BRM_TRY_MTX(sc.alloc(&hist, (size_t)rblk * 256 * 4));
        BRM_TRY_MTX(sc.alloc(&off, ((size_t)rblk * 256 + 1) * 8));
        BRM_TRY_MTX(sc.alloc(&rtmp, scan_tmp_bytes(rblk * 256)));
        for (int p = 0; p < npass; p++) {
            k_rs_hist<<<rblk, kRsThreads, 0, s>>>(k0, n, 8 * p, rblk, hist);
            count_launch();
            launch_scan_i64(hist, off, rblk * 256, rtmp, s);
            k_rs_scatter<<<rblk, kRsThreads, 0, s>>>(k0, v0, n, 8 * p, rblk, off, k1, v1);
            count_launch();
            std::swap(k0, k1);
            std::swap(v0, v1);
        }
    }
    int *rpt = nullptr, *col = nullptr;
    void *val = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&rpt, 4 * ((size_t)M + 1), s);
    if (e == cudaSuccess)
        e = cudaMallocAsync((void **)&col, 4 * (size_t)n, s);
    if (e == cudaSuccess)
        e = cudaMallocAsync(&val, (dtype == BRM_F64 ? 8 : 4) * (size_t)n, s);
    auto drop = [&]() {
        if (rpt)
            cudaFreeAsync(rpt, s);
        if (col)
            cudaFreeAsync(col, s);
        if (val)
            cudaFreeAsync(val, s);
    };
    if (e != cudaSuccess) {
        drop();
        return cuda_st(e);
    }
    const int cgrid = (int)std::min<long long>((n + 255) / 256, (long long)num_sms * 16);
    if (dtype == BRM_F64)
        k_mtx_csr<double><<<cgrid, 256, 0, s>>>(k0, v0, n, cb, M, rpt, col, (double *)val, dcnt);
    else
        k_mtx_csr<float><<<cgrid, 256, 0, s>>>(k0, v0, n, cb, M, rpt, col, (float *)val, dcnt);
    count_launch();
    e = cudaMemcpyAsync(&hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || hc.err) {
        drop();
        return e != cudaSuccess ? cuda_st(e) : BRM_ERR_FORMAT;
    }
    const double t3 = now_s();
    out->M = M;
    out->N = N;
    out->nnz = n;
    out->rpt = rpt;
    out->col = col;
    out->val = val;
    if (tm) {
        tm->read = t1 - t0;
        tm->parse = t2 - t1;
        tm->build = t3 - t2;
        tm->total = t3 - t0;
    }
    return BRM_SUCCESS;
}

}  // namespace
}  // namespace brm

extern "C" {

int brm_read_mtx_device(brm_context ctx, brm_dtype dtype, const char *path, int *M, int *N,
                        int *nnz, int **rpt, int **col, void **val, brm_mtx_timing *timing)
{
    if (!ctx || !path || !M || !N || !nnz || !rpt || !col || !val)
        return BRM_ERR_INVALID_VALUE;
    if (dtype != BRM_F64 && dtype != BRM_F32)
        return BRM_ERR_INVALID_VALUE;
    brm::ReadOut o;
    const int st = brm::read_device(path, dtype, brm::context_stream(ctx),
                                    brm::context_num_sms(ctx), &o, timing);
    if (st != BRM_SUCCESS)
        return st;
    *M = o.M;
    *N = o.N;
    *nnz = o.nnz;
    *rpt = o.rpt;
    *col = o.col;
    *val = o.val;
    return BRM_SUCCESS;
}

int brm_read_mtx(const char *path, brm_dtype dtype, int *M, int *N, int *nnz, int **rpt,
                 int **col, void **val, brm_mtx_timing *timing)
{
    if (!path || !M || !N || !nnz || !rpt || !col || !val)
        return BRM_ERR_INVALID_VALUE;
    if (dtype != BRM_F64 && dtype != BRM_F32)
        return BRM_ERR_INVALID_VALUE;
    std::lock_guard<std::mutex> lock(brm::shared_context_mutex());
    brm_context ctx = nullptr;
    int st = brm::shared_context(&ctx);
    if (st != BRM_SUCCESS)
        return st;
    cudaStream_t s = brm::context_stream(ctx);
    brm::ReadOut o;
    const double t0 = brm::now_s();
    st = brm::read_device(path, dtype, s, brm::context_num_sms(ctx), &o, timing);
    if (st != BRM_SUCCESS)
        return st;
    const size_t vb = dtype == BRM_F64 ? 8 : 4;
    int *hr = (int *)brm::host_alloc(4 * ((size_t)o.M + 1));
    int *hc = (int *)brm::host_alloc(4 * (size_t)(o.nnz > 0 ? o.nnz : 1));
    void *hv = brm::host_alloc(vb * (size_t)(o.nnz > 0 ? o.nnz : 1));
    cudaError_t e = (hr && hc && hv) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hr, o.rpt, 4 * ((size_t)o.M + 1), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hc, o.col, 4 * (size_t)o.nnz, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hv, o.val, vb * (size_t)o.nnz, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(o.rpt, s);
    cudaFreeAsync(o.col, s);
    cudaFreeAsync(o.val, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        brm_free(hr);
        brm_free(hc);
        brm_free(hv);
        return brm::cuda_st(e);
    }
    *M = o.M;
    *N = o.N;
    *nnz = o.nnz;
    *rpt = hr;
    *col = hc;
    *val = hv;
    if (timing)
        timing->total = brm::now_s() - t0;
    return BRM_SUCCESS;
}

}  // extern "C"
