// Deterministic synthetic CSR generators (see include/brm_gen.h).
#include "brm_gen.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

// splitmix64 (Steele, Lea, Flood 2014) to expand a seed into PRNG state.
inline uint64_t splitmix64(uint64_t &x)
{
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// xoshiro256** (Blackman and Vigna 2018).
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed, uint64_t stream = 0)
    {
        uint64_t x = seed ^ (stream * 0xd1b54a32d192ed03ULL);
        for (auto &w : s)
            w = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    inline uint64_t next()
    {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform double in [0, 1) with 53 random bits
    inline double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    // uniform integer in [0, n) by multiply-shift
    inline uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
    inline double sym(double h) { return (2.0 * uniform() - 1.0) * h; }
    double normal()
    {
        // Box-Muller; u1 in (0,1]
        double u1 = 1.0 - uniform();
        double u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

bool alloc_csr(brm_host_csr *out, int M, int N, long long nnz)
{
    std::memset(out, 0, sizeof(*out));
    if (nnz > 2147483647LL)
        return false;
    out->M = M;
    out->N = N;
    out->nnz = (int)nnz;
    out->rpt = (int *)std::malloc(sizeof(int) * ((size_t)M + 1));
    out->col = (int *)std::malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    out->val = (double *)std::malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    if (!out->rpt || !out->col || !out->val) {
        brm_host_csr_free(out);
        return false;
    }
    return true;
}

// k distinct values in [0, n), sorted (Floyd's sampling when k is small
// relative to n, a shuffled prefix otherwise).
void sample_distinct(Rng &rng, int n, int k, std::vector<int> &outv, std::vector<char> &mark)
{
    outv.clear();
    if (k <= 0)
        return;
    if ((long long)k * 4 >= n) {
        std::vector<int> all(n);
        for (int i = 0; i < n; i++)
            all[i] = i;
        for (int i = 0; i < k; i++) {
            int j = i + (int)rng.below((uint32_t)(n - i));
            std::swap(all[i], all[j]);
        }
        outv.assign(all.begin(), all.begin() + k);
    } else {
        // Floyd: for j in n-k .. n-1 pick t in [0, j]; take t unless taken, else j.
        if ((int)mark.size() < n)
            mark.assign(n, 0);
        for (int j = n - k; j < n; j++) {
            int t = (int)rng.below((uint32_t)(j + 1));
            int pick = mark[t] ? j : t;
            mark[pick] = 1;
            outv.push_back(pick);
        }
        for (int v : outv)
            mark[v] = 0;
    }
    std::sort(outv.begin(), outv.end());
}

}  // namespace

extern "C" {

void brm_host_csr_free(brm_host_csr *m)
{
    if (!m)
        return;
    std::free(m->rpt);
    std::free(m->col);
    std::free(m->val);
    m->rpt = nullptr;
    m->col = nullptr;
    m->val = nullptr;
}

int brm_gen_er(int n, int per_row, unsigned long long seed, brm_host_csr *out)
{
    if (n <= 0 || per_row < 0 || per_row > n || !out)
        return 1;
    if (!alloc_csr(out, n, n, (long long)n * per_row))
        return 3;
    Rng rng(seed, 1), vr(seed, 2);
    std::vector<int> cols;
    std::vector<char> mark;
    out->rpt[0] = 0;
    for (int i = 0; i < n; i++) {
        sample_distinct(rng, n, per_row, cols, mark);
        int base = i * per_row;
        for (int j = 0; j < per_row; j++) {
            out->col[base + j] = cols[j];
            out->val[base + j] = vr.sym(1.0);
        }
        out->rpt[i + 1] = base + per_row;
    }
    return 0;
}

int brm_gen_rmat(int scale, long long edges, double a, double b, double c,
                 unsigned long long seed, brm_host_csr *out)
{
    if (scale < 1 || scale > 30 || edges < 0 || !out || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return 1;
    const int n = 1 << scale;
    std::vector<uint64_t> keys((size_t)edges);
    Rng rng(seed, 3);
    const double ab = a + b, abc = a + b + c;
    for (long long e = 0; e < edges; e++) {
        uint32_t r = 0, cc = 0;
        for (int bit = scale - 1; bit >= 0; bit--) {
            double u = rng.uniform();
            uint32_t rb = u >= ab ? 1u : 0u;                             // quadrants c, d
            uint32_t cb = ((u >= a && u < ab) || u >= abc) ? 1u : 0u;    // quadrants b, d
            r |= rb << bit;
            cc |= cb << bit;
        }
        keys[(size_t)e] = ((uint64_t)r << 32) | cc;
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    if (!alloc_csr(out, n, n, (long long)keys.size()))
        return 3;
    std::memset(out->rpt, 0, sizeof(int) * ((size_t)n + 1));
    Rng vr(seed, 4);
    for (size_t e = 0; e < keys.size(); e++) {
        out->rpt[(keys[e] >> 32) + 1]++;
        out->col[e] = (int)(keys[e] & 0xffffffffu);
        out->val[e] = vr.sym(1.0);
    }
    for (int i = 0; i < n; i++)
        out->rpt[i + 1] += out->rpt[i];
    return 0;
}

int brm_gen_stencil27(int nx, int ny, int nz, double jitter, unsigned long long seed,
                      brm_host_csr *out)
{
    if (nx <= 0 || ny <= 0 || nz <= 0 || !out)
        return 1;
    long long n = (long long)nx * ny * nz;
    if (n > 2147483647LL)
        return 1;
    auto cnt = [](int x, int nxx) { return (x > 0) + 1 + (x < nxx - 1); };
    long long nnz = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++)
                nnz += (long long)cnt(x, nx) * cnt(y, ny) * cnt(z, nz);
    if (!alloc_csr(out, (int)n, (int)n, nnz))
        return 3;
    Rng vr(seed, 5);
    long long p = 0;
    int row = 0;
    out->rpt[0] = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++, row++) {
                for (int dz = -1; dz <= 1; dz++) {
                    int zz = z + dz;
                    if (zz < 0 || zz >= nz) continue;
                    for (int dy = -1; dy <= 1; dy++) {
                        int yy = y + dy;
                        if (yy < 0 || yy >= ny) continue;
                        for (int dx = -1; dx <= 1; dx++) {
                            int xx = x + dx;
                            if (xx < 0 || xx >= nx) continue;
                            int colx = (zz * ny + yy) * nx + xx;
                            double v = (colx == row) ? 26.0 : -1.0;
                            out->col[p] = colx;
                            out->val[p] = v + vr.sym(jitter);
                            p++;
                        }
                    }
                }
                out->rpt[row + 1] = (int)p;
            }
    return 0;
}

int brm_gen_lognormal(int M, int N, double mu, double sigma, int cap,
                      unsigned long long seed, brm_host_csr *out)
{
    if (M < 0 || N <= 0 || cap < 0 || !out)
        return 1;
    Rng lr(seed, 6);
    std::vector<int> len(M);
    long long nnz = 0;
    int hi = std::min(cap, N);
    for (int i = 0; i < M; i++) {
        double x = std::exp(mu + sigma * lr.normal());
        long long k = (long long)std::floor(x + 0.5);
        if (k > hi) k = hi;
        if (k < 0) k = 0;
        len[i] = (int)k;
        nnz += k;
    }
    if (!alloc_csr(out, M, N, nnz))
        return 3;
    Rng rng(seed, 7), vr(seed, 8);
    std::vector<int> cols;
    std::vector<char> mark;
    out->rpt[0] = 0;
    int p = 0;
    for (int i = 0; i < M; i++) {
        sample_distinct(rng, N, len[i], cols, mark);
        for (int v : cols) {
            out->col[p] = v;
            out->val[p] = vr.sym(1.0);
            p++;
        }
        out->rpt[i + 1] = p;
    }
    return 0;
}

int brm_gen_uniform(int M, int N, int max_per_row, unsigned long long seed, brm_host_csr *out)
{
    if (M < 0 || N <= 0 || max_per_row < 0 || !out)
        return 1;
    Rng lr(seed, 9);
    std::vector<int> len(M);
    long long nnz = 0;
    int hi = std::min(max_per_row, N);
    for (int i = 0; i < M; i++) {
        len[i] = (int)lr.below((uint32_t)hi + 1);
        nnz += len[i];
    }
    if (!alloc_csr(out, M, N, nnz))
        return 3;
    Rng rng(seed, 10), vr(seed, 11);
    std::vector<int> cols;
    std::vector<char> mark;
    out->rpt[0] = 0;
    int p = 0;
    for (int i = 0; i < M; i++) {
        sample_distinct(rng, N, len[i], cols, mark);
        for (int v : cols) {
            out->col[p] = v;
            out->val[p] = vr.sym(1.0);
            p++;
        }
        out->rpt[i + 1] = p;
    }
    return 0;
}

}  // extern "C"
