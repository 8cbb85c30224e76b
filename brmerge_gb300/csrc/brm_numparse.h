// brm_numparse.h -- MatrixMarket token parsing, shared by the device reader
// and a host copy used to test it.
//
// Tokens follow C++ stream extraction in the "C" locale, which is how the
// reference reads a MatrixMarket body (BRMerge-SpGEMM/src/CSR.cpp:297-335):
// integers [+-]?[0-9]+ within int32, reals
// [+-]?([0-9]+(.[0-9]*)?|.[0-9]+)([eE][+-]?[0-9]+)?, converted with correct
// rounding (round to nearest, ties to even).  Decimal to binary conversion:
//   * Clinger's fast path (W. D. Clinger, "How to read floating point
//     numbers accurately", PLDI 1990): significand w <= 2^53 and decimal
//     exponent |q| <= 22 -> one IEEE multiply or divide of exact operands;
//   * otherwise Eisel-Lemire (D. Lemire, "Number parsing at a gigabyte per
//     second", Software: Practice and Experience 51(8), 2021) with the 128-bit
//     truncated powers of five of brm_pow5.h: w * T(q) from 64x64-bit
//     products, refused whenever the truncation could change the rounding;
//   * a refused token, a subnormal or overflowing result, or more than 19
//     significant digits whose two bracketing conversions disagree is left
//     to an exact conversion (strtod) by the caller.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

#include "brm_pow5.h"

namespace brm {

enum TokStatus : int { kTokOk = 0, kTokSlow = 1, kTokBad = -1 };

__host__ __device__ inline bool tok_space(unsigned c)
{
    // isspace in the "C" locale
    return c == ' ' || (c >= 9 && c <= 13);
}

__host__ __device__ inline bool tok_digit(unsigned c) { return c - '0' < 10u; }

// Byte accessor over a contiguous token.
struct TokPtr {
    const unsigned char *p;
    __host__ __device__ unsigned operator()(int i) const { return p[i]; }
};

// [+-]?[0-9]+ within int32; `at(i)` returns byte i of the token.
template <typename Get>
__host__ __device__ inline int parse_int_at(const Get &at, int len, long long *out)
{
    int i = 0;
    bool neg = false;
    if (i < len && (at(i) == '+' || at(i) == '-')) {
        neg = at(i) == '-';
        i++;
    }
    if (i >= len)
        return kTokBad;
    long long v = 0;
    for (; i < len; i++) {
        const unsigned c = at(i);
        if (!tok_digit(c))
            return kTokBad;
        v = v * 10 + (c - '0');
        if (v > 2147483648ll)
            return kTokBad;
    }
    v = neg ? -v : v;
    if (v > 2147483647ll)
        return kTokBad;
    *out = v;
    return kTokOk;
}

__host__ __device__ inline int parse_int_tok(const unsigned char *p, int len, long long *out)
{
    return parse_int_at(TokPtr{p}, len, out);
}

__host__ __device__ inline uint64_t mul_hi64(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

__host__ __device__ inline int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

__host__ __device__ inline double bits_to_double(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    __builtin_memcpy(&d, &b, 8);
    return d;
#endif
}

// Eisel-Lemire: w != 0, q in [kPow5Min, kPow5Max].  Returns false when the
// 128-bit approximation cannot decide the rounding, or the result is
// subnormal or overflows.  `pow5` is the table of brm_pow5.h.
__host__ __device__ inline bool eisel_lemire(uint64_t w, int q, const uint64_t (*pow5)[2],
                                             uint64_t *bits)
{
    const int lz = clz64(w);
    w <<= lz;
    const uint64_t thi = pow5[q - kPow5Min][0], tlo = pow5[q - kPow5Min][1];
    uint64_t xhi = mul_hi64(w, thi), xlo = w * thi;
    // the product of w with the low half of T(q) adds less than w to xlo
    if ((xhi & 0x1FF) == 0x1FF && xlo + w < xlo) {
        const uint64_t yhi = mul_hi64(w, tlo), ylo = w * tlo;
        uint64_t mhi = xhi, mlo = xlo + yhi;
        if (mlo < xlo)
            mhi++;
        if ((mhi & 0x1FF) == 0x1FF && mlo + 1 == 0 && ylo + w < ylo)
            return false;
        xhi = mhi;
        xlo = mlo;
    }
    const int msb = (int)(xhi >> 63);
    uint64_t m = xhi >> (msb + 9);
    // biased exponent: floor(q log2 10) + 1086 - lz + msb
    long long be = (long long)((217706 * q) >> 16) + 1086 - lz + msb;
    if (xlo == 0 && (xhi & 0x1FF) == 0 && (m & 3) == 1)
        return false;  // exactly halfway as far as 128 bits can tell
    m += m & 1;
    m >>= 1;
    if (m >> 53) {
        m >>= 1;
        be++;
    }
    if (be < 1 || be > 0x7FE)
        return false;
    *bits = ((uint64_t)be << 52) | (m & ((1ull << 52) - 1));
    return true;
}

// A real token.  kTokOk: *out holds the correctly rounded value; kTokSlow:
// the grammar is valid but the value needs an exact conversion; kTokBad: not
// a real number.  pow5 == nullptr checks the grammar only (kTokSlow when
// valid).
template <typename Get>
__host__ __device__ inline int parse_real_at(const Get &at, int len, const uint64_t (*pow5)[2],
                                             double *out)
{
    int i = 0;
    bool neg = false;
    if (i < len && (at(i) == '+' || at(i) == '-')) {
        neg = at(i) == '-';
        i++;
    }
    uint64_t w = 0;
    int nd = 0;        // significant digits kept in w (at most 19)
    long long q = 0;   // decimal exponent of w
    int ndig = 0;      // mantissa digits seen
    bool trunc = false;  // a nonzero digit beyond the 19 kept
    for (; i < len && tok_digit(at(i)); i++) {
        const unsigned d = at(i) - '0';
        ndig++;
        if (nd == 0 && d == 0)
            continue;
        if (nd < 19) {
            w = w * 10 + d;
            nd++;
        } else {
            q++;
            trunc |= d != 0;
        }
    }
    if (i < len && at(i) == '.') {
        i++;
        for (; i < len && tok_digit(at(i)); i++) {
            const unsigned d = at(i) - '0';
            ndig++;
            if (nd == 0 && d == 0) {
                q--;
                continue;
            }
            if (nd < 19) {
                w = w * 10 + d;
                nd++;
                q--;
            } else {
                trunc |= d != 0;
            }
        }
    }
    if (ndig == 0)
        return kTokBad;
    if (i < len && (at(i) == 'e' || at(i) == 'E')) {
        i++;
        bool eneg = false;
        if (i < len && (at(i) == '+' || at(i) == '-')) {
            eneg = at(i) == '-';
            i++;
        }
        long long ev = 0;
        int ed = 0;
        for (; i < len && tok_digit(at(i)); i++, ed++)
            if (ev < 1000000)
                ev = ev * 10 + (at(i) - '0');
        if (ed == 0)
            return kTokBad;
        q += eneg ? -ev : ev;
    }
    if (i != len)
        return kTokBad;
    if (!pow5)
        return kTokSlow;
    if (w == 0) {
        *out = neg ? -0.0 : 0.0;
        return kTokOk;
    }
    double v;
    if (!trunc && w <= (1ull << 53) && q >= -22 && q <= 22) {
        // exact powers of ten: 10^0 .. 10^22 are doubles
        double p10 = 1.0;
        for (int k = 0; k < (q < 0 ? -q : q); k++)
            p10 *= 10.0;
#ifdef __CUDA_ARCH__
        v = q < 0 ? __ddiv_rn((double)w, p10) : __dmul_rn((double)w, p10);
#else
        v = q < 0 ? (double)w / p10 : (double)w * p10;
#endif
    } else {
        if (q < kPow5Min || q > kPow5Max)
            return kTokSlow;
        uint64_t b0;
        if (!eisel_lemire(w, (int)q, pow5, &b0))
            return kTokSlow;
        if (trunc) {
            // the value lies in (w, w + 1) * 10^q: both ends must agree
            uint64_t b1;
            if (!eisel_lemire(w + 1, (int)q, pow5, &b1) || b1 != b0)
                return kTokSlow;
        }
        v = bits_to_double(b0);
    }
    *out = neg ? -v : v;
    return kTokOk;
}

__host__ __device__ inline int parse_real_tok(const unsigned char *p, int len,
                                              const uint64_t (*pow5)[2], double *out)
{
    return parse_real_at(TokPtr{p}, len, pow5, out);
}

}  // namespace brm
