// brm_common.cuh -- shared device helpers for the BRMerge SpGEMM kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace brm {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// Value arithmetic with explicit IEEE round-to-nearest and no contraction:
// the merge order fixes every rounding, so products and sums stay separate.
__device__ __forceinline__ double vmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double vadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(kFull, v, o);
        if (lane >= o)
            v += n;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(kFull, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T n = __shfl_xor_sync(kFull, v, o);
        v = n > v ? n : v;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_min(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T n = __shfl_xor_sync(kFull, v, o);
        v = n < v ? n : v;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread.  `ws` is shared
// scratch of NT/32+1 entries.  Returns the exclusive prefix; *total gets
// the block sum.  Contains three __syncthreads().
template <int NT, typename T>
__device__ __forceinline__ T block_excl_scan(T v, T *ws, T *total)
{
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T inc = warp_incl_scan(v);
    __syncthreads();  // ws may still be read by a previous block-wide call
    if (lane == 31)
        ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        T s = lane < NW ? ws[lane] : T(0);
        T si = warp_incl_scan(s);
        if (lane < NW)
            ws[lane] = si - s;
        if (lane == NW - 1)
            ws[NW] = si;
    }
    __syncthreads();
    T r = ws[w] + inc - v;
    *total = ws[NW];
    return r;
}

// Asynchronous 16-byte global -> shared copy (cp.async, cached in L2 only);
// both addresses 16-byte aligned.  cp_async_wait_all waits for every copy
// this thread has issued.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem_src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <int NT, typename T>
__device__ __forceinline__ T block_sum(T v, T *ws)
{
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T s = warp_sum(v);
    __syncthreads();
    if (lane == 0)
        ws[w] = s;
    __syncthreads();
    T t = T(0);
    for (int i = 0; i < NW; i++)
        t += ws[i];
    return t;
}

template <int NT, typename T>
__device__ __forceinline__ T block_max(T v, T *ws)
{
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T s = warp_max(v);
    __syncthreads();
    if (lane == 0)
        ws[w] = s;
    __syncthreads();
    T t = ws[0];
    for (int i = 1; i < NW; i++)
        t = ws[i] > t ? ws[i] : t;
    return t;
}

template <int NT, typename T>
__device__ __forceinline__ T block_min(T v, T *ws)
{
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T s = warp_min(v);
    __syncthreads();
    if (lane == 0)
        ws[w] = s;
    __syncthreads();
    T t = ws[0];
    for (int i = 1; i < NW; i++)
        t = ws[i] < t ? ws[i] : t;
    return t;
}

// Split level of two distinct leaves of the binary merge tree: the tree
// level (0-based) at which leaves a and b are combined minus one, i.e. the
// index of the highest differing bit.
__device__ __forceinline__ int split_level(int a, int b) { return 31 - __clz(a ^ b); }

// Order-exact reduction of one column's contributions.
//
// The reference merges the k lists of a row pairwise, adjacent pairs first
// (BRMerge-SpGEMM/inc/spgemm.h:639-707): list l of level L+1 is the merge of
// lists 2l and 2l+1 of level L, an odd last list passes through, and equal
// columns are added as left + right (:651-653).  For one column that is a
// binary trie over the leaf index l: siblings combine as left + right and a
// node with one present child passes that child's value through unchanged.
// ShiftReduce evaluates that trie for leaves presented in increasing order:
// consecutive leaves a < b are joined at split_level(a, b), and a lower split
// binds tighter (operator-precedence parsing).  The stack holds at most one
// entry per tree level.
template <typename T, int DEPTH = 33>
struct ShiftReduce {
    T val[DEPTH];
    int op[DEPTH];  // op[i] = split level between entries i and i+1
    int n;
    int last;
    __device__ __forceinline__ void init(int leaf, T v)
    {
        val[0] = v;
        n = 1;
        last = leaf;
    }
    __device__ __forceinline__ void push(int leaf, T v)
    {
        int s = split_level(last, leaf);
        while (n >= 2 && op[n - 2] < s) {
            val[n - 2] = vadd(val[n - 2], val[n - 1]);
            n--;
        }
        op[n - 1] = s;
        val[n] = v;
        n++;
        last = leaf;
    }
    __device__ __forceinline__ T finish()
    {
        while (n >= 2) {
            val[n - 2] = vadd(val[n - 2], val[n - 1]);
            n--;
        }
        return val[0];
    }
};

// Closed forms of the trie for three and four leaves in increasing order.
// Adjacent leaves a < b join at split_level(a, b); the highest adjacent split
// is the root, and two adjacent pairs never share a split level when every
// split between them is lower, so the maximum is unique.
template <typename T>
__device__ __forceinline__ T trie3(int l0, int l1, int l2, T v0, T v1, T v2)
{
    return split_level(l0, l1) < split_level(l1, l2) ? vadd(vadd(v0, v1), v2)
                                                     : vadd(v0, vadd(v1, v2));
}

template <typename T>
__device__ __forceinline__ T trie4(int l0, int l1, int l2, int l3, T v0, T v1, T v2, T v3)
{
    const int s01 = split_level(l0, l1), s12 = split_level(l1, l2), s23 = split_level(l2, l3);
    if (s12 > s01 && s12 > s23)
        return vadd(vadd(v0, v1), vadd(v2, v3));
    if (s01 > s23)
        return vadd(v0, s12 < s23 ? vadd(vadd(v1, v2), v3) : vadd(v1, vadd(v2, v3)));
    return vadd(s01 < s12 ? vadd(vadd(v0, v1), v2) : vadd(v0, vadd(v1, v2)), v3);
}

// Orders two (leaf, value) pairs by leaf.
template <typename T>
__device__ __forceinline__ void leaf_cas(int &la, T &va, int &lb, T &vb)
{
    if (la > lb) {
        const int l = la;
        la = lb;
        lb = l;
        const T v = va;
        va = vb;
        vb = v;
    }
}

// Sorts eight (leaf, value) pairs by leaf in registers (Batcher's odd-even
// merge network, 19 comparators).
template <typename T>
__device__ __forceinline__ void leaf_sort8(int (&l)[8], T (&v)[8])
{
    leaf_cas(l[0], v[0], l[1], v[1]);
    leaf_cas(l[2], v[2], l[3], v[3]);
    leaf_cas(l[4], v[4], l[5], v[5]);
    leaf_cas(l[6], v[6], l[7], v[7]);
    leaf_cas(l[0], v[0], l[2], v[2]);
    leaf_cas(l[1], v[1], l[3], v[3]);
    leaf_cas(l[4], v[4], l[6], v[6]);
    leaf_cas(l[5], v[5], l[7], v[7]);
    leaf_cas(l[1], v[1], l[2], v[2]);
    leaf_cas(l[5], v[5], l[6], v[6]);
    leaf_cas(l[0], v[0], l[4], v[4]);
    leaf_cas(l[1], v[1], l[5], v[5]);
    leaf_cas(l[2], v[2], l[6], v[6]);
    leaf_cas(l[3], v[3], l[7], v[7]);
    leaf_cas(l[2], v[2], l[4], v[4]);
    leaf_cas(l[3], v[3], l[5], v[5]);
    leaf_cas(l[1], v[1], l[2], v[2]);
    leaf_cas(l[3], v[3], l[4], v[4]);
    leaf_cas(l[5], v[5], l[6], v[6]);
}

// ShiftReduce with its stack in registers for at most D leaves: the entry
// below the top is always st[0], so every access uses a fixed index (a push
// shifts the stack down, a reduction shifts it up).
template <typename T, int D>
struct RegShiftReduce {
    T st[D - 1];
    int op[D - 1];  // op[i]: split level between st[i] and the entry above it
    int nb;         // entries below the top
    T cur;          // top of the stack
    int last;
    __device__ __forceinline__ void init(int leaf, T v)
    {
        nb = 0;
        cur = v;
        last = leaf;
    }
    __device__ __forceinline__ void pop()
    {
        cur = vadd(st[0], cur);
#pragma unroll
        for (int i = 0; i < D - 2; i++) {
            st[i] = st[i + 1];
            op[i] = op[i + 1];
        }
        nb--;
    }
    __device__ __forceinline__ void push(int leaf, T v)
    {
        const int s = split_level(last, leaf);
        while (nb > 0 && op[0] < s)
            pop();
#pragma unroll
        for (int i = D - 2; i > 0; i--) {
            st[i] = st[i - 1];
            op[i] = op[i - 1];
        }
        st[0] = cur;
        op[0] = s;
        nb++;
        cur = v;
        last = leaf;
    }
    __device__ __forceinline__ T finish()
    {
        while (nb > 0)
            pop();
        return cur;
    }
};

// Trie value of n <= 32 leaves held one per lane (lane j < n holds the j-th
// smallest leaf and its value); called by a full warp, result in lane 0.
// Each round joins every adjacent pair of surviving subtrees whose split
// level is the lowest present: such pairs are disjoint siblings, and a
// subtree is represented by any of its leaves.
template <typename T>
__device__ __forceinline__ T warp_trie(int leaf, T v, int n)
{
    const int lane = threadIdx.x & 31;
    bool alive = lane < n;
    for (;;) {
        const unsigned am = __ballot_sync(kFull, alive);
        if ((am & (am - 1u)) == 0)
            break;
        const unsigned after = am & ~((2u << lane) - 1u);
        const int nl = after ? __ffs(after) - 1 : lane;
        const int kn = __shfl_sync(kFull, leaf, nl);
        const T vn = __shfl_sync(kFull, v, nl);
        const bool has = alive && after != 0u;
        const int s = has ? split_level(leaf, kn) : 64;
        const int smin = __reduce_min_sync(kFull, s);
        const bool comb = has && s == smin;
        if (comb)
            v = vadd(v, vn);
        const unsigned cm = __ballot_sync(kFull, comb);
        const unsigned before = am & ((1u << lane) - 1u);
        if (alive && before && ((cm >> (31 - __clz(before))) & 1u))
            alive = false;
    }
    return v;
}

}  // namespace brm
