// Software IEEE-754 binary128 (round-to-nearest-even) for the few operations
// of the reference's real(16) resampling recurrence: conversion from double
// and from integers, add, subtract, multiply, divide and floor.  Normal
// numbers and zero are handled exactly; the recurrence never produces
// subnormals, infinities or NaNs (its values stay within [2^-1100, 2^40]).
// Usable on host and device; the host build is checked against GCC's
// __float128 in the test suite.
#pragma once
#include <stdint.h>

#ifndef SMC_HD
#ifdef __CUDACC__
#define SMC_HD __host__ __device__ __forceinline__
#else
#define SMC_HD inline
#endif
#endif

namespace smc {

typedef unsigned __int128 u128;

struct q128 {
    int sign;   // 0 or 1
    int exp;    // unbiased exponent of the leading bit
    u128 man;   // 113-bit significand with the leading bit set; 0 for zero
};

SMC_HD q128 q128_zero() { return {0, 0, 0}; }

SMC_HD int clz128(u128 x) {
    uint64_t hi = (uint64_t)(x >> 64), lo = (uint64_t)x;
#ifdef __CUDA_ARCH__
    if (hi) return __clzll((long long)hi);
    if (lo) return 64 + __clzll((long long)lo);
    return 128;
#else
    if (hi) return __builtin_clzll(hi);
    if (lo) return 64 + __builtin_clzll(lo);
    return 128;
#endif
}

// Round a significand carrying `extra` bits below the 113 kept bits (plus a
// separate sticky flag) to nearest-even and build the number.
SMC_HD q128 q128_round(int sign, int exp, u128 m, int extra, bool sticky) {
    // m has its leading bit at position 112 + extra
    u128 keep = m >> extra;
    u128 rem = extra ? (m & ((((u128)1) << extra) - 1)) : 0;
    u128 half = extra ? ((u128)1) << (extra - 1) : 0;
    bool up = extra > 0 && (rem > half || (rem == half && (sticky || (keep & 1))));
    if (up) {
        keep += 1;
        if (keep >> 113) { keep >>= 1; exp += 1; }
    }
    return {sign, exp, keep};
}

// Normalise an arbitrary nonzero integer significand m * 2^(e0) so that the
// result carries 113 bits, then round.
SMC_HD q128 q128_from_scaled(int sign, u128 m, int e0, bool sticky_in) {
    if (m == 0) return q128_zero();
    int lead = 127 - clz128(m);          // position of the leading bit
    int exp = e0 + lead;                  // value = m * 2^e0
    if (lead > 112) {
        int extra = lead - 112;
        return q128_round(sign, exp, m, extra, sticky_in);
    }
    (void)sticky_in;  // exact significands only reach this branch
    return {sign, exp, m << (112 - lead)};
}

SMC_HD q128 q128_from_double(double d) {
    if (d == 0.0) return q128_zero();
    union { double d; uint64_t u; } c;
    c.d = d;
    int sign = (int)(c.u >> 63);
    int be = (int)((c.u >> 52) & 0x7ff);
    uint64_t frac = c.u & 0xfffffffffffffull;
    u128 m;
    int e0;
    if (be == 0) { m = frac; e0 = -1074; }            // subnormal double
    else { m = frac | (1ull << 52); e0 = be - 1075; }
    return q128_from_scaled(sign, m, e0, false);
}

SMC_HD q128 q128_from_int(long long v) {
    if (v == 0) return q128_zero();
    int sign = v < 0;
    unsigned long long a = sign ? (unsigned long long)(-(v + 1)) + 1ull : (unsigned long long)v;
    return q128_from_scaled(sign, (u128)a, 0, false);
}

// shift right with sticky
SMC_HD u128 shr_sticky(u128 m, int s, bool &sticky) {
    if (s <= 0) return m;
    if (s >= 128) { sticky = sticky || (m != 0); return 0; }
    u128 lost = m & ((((u128)1) << s) - 1);
    if (lost) sticky = true;
    return m >> s;
}

SMC_HD q128 q128_add(q128 a, q128 b) {
    if (a.man == 0) return b;
    if (b.man == 0) return a;
    // work with 3 guard bits: significands scaled to leading bit 115
    if (a.exp < b.exp || (a.exp == b.exp && a.man < b.man)) { q128 t = a; a = b; b = t; }
    u128 ma = a.man << 3, mb = b.man << 3;
    bool sticky = false;
    mb = shr_sticky(mb, a.exp - b.exp, sticky);
    int e0 = a.exp - 115;
    if (a.sign == b.sign) {
        u128 s = ma + mb;  // leading bit at 115 or 116
        int lead = 127 - clz128(s);
        return q128_round(a.sign, e0 + lead, s, lead - 112, sticky);
    } else {
        // |a| >= |b|; subtract; a sticky bit of b means the true difference is
        // slightly smaller than ma - mb
        u128 d = ma - mb;
        if (sticky) d -= 1;  // borrow of the discarded bits; sticky stays set
        if (d == 0 && !sticky) return q128_zero();
        int lead = 127 - clz128(d);
        int exp = e0 + lead;
        if (lead >= 112) return q128_round(a.sign, exp, d, lead - 112, sticky);
        // large cancellation: exact when the shift happened by <= 1 (no sticky)
        return {a.sign, exp, d << (112 - lead)};
    }
}

SMC_HD q128 q128_neg(q128 a) { a.sign ^= (a.man != 0); return a; }
SMC_HD q128 q128_sub(q128 a, q128 b) { return q128_add(a, q128_neg(b)); }

SMC_HD q128 q128_mul(q128 a, q128 b) {
    if (a.man == 0 || b.man == 0) return q128_zero();
    int sign = a.sign ^ b.sign;
    uint64_t ah = (uint64_t)(a.man >> 64), al = (uint64_t)a.man;
    uint64_t bh = (uint64_t)(b.man >> 64), bl = (uint64_t)b.man;
    u128 ll = (u128)al * bl, lh = (u128)al * bh, hl = (u128)ah * bl, hh = (u128)ah * bh;
    // 256-bit product P = hh*2^128 + (lh+hl)*2^64 + ll
    u128 mid = lh + hl;                       // < 2^114, no overflow
    u128 lo = ll + (mid << 64);
    u128 carry = lo < ll ? 1 : 0;
    u128 hi = hh + (mid >> 64) + carry;
    // product has its leading bit at 224 or 225 -> hi has it at 96 or 97
    int lead_hi = 127 - clz128(hi);           // 96 or 97
    int shift = lead_hi + 128 - 112;          // bits to drop from the 256-bit value
    // keep = P >> shift, with rounding bits: take P >> (shift - 3) into 116+ bits
    int s = shift - 3;                        // 109 or 110 (< 128)
    u128 top = (hi << (128 - s)) | (lo >> s);
    bool sticky = (lo & ((((u128)1) << s) - 1)) != 0;
    int exp = a.exp + b.exp + (lead_hi + 128 - 224);
    return q128_round(sign, exp, top, 3, sticky);
}

SMC_HD q128 q128_div(q128 a, q128 b) {
    if (a.man == 0) return q128_zero();
    int sign = a.sign ^ b.sign;
    u128 r = a.man, d = b.man, q = 0;
    int exp = a.exp - b.exp;
    if (r < d) { r <<= 1; exp -= 1; }
    // 113 quotient bits + 3 rounding bits
    for (int i = 0; i < 116; ++i) {
        q <<= 1;
        if (r >= d) { r -= d; q |= 1; }
        r <<= 1;
    }
    return q128_round(sign, exp, q, 3, r != 0);
}

// floor to a 64-bit integer (|value| < 2^62)
SMC_HD long long q128_floor(q128 a) {
    if (a.man == 0) return 0;
    if (a.exp < 0) return a.sign ? -1 : 0;
    int sh = 112 - a.exp;
    u128 ip = sh > 0 ? (a.man >> sh) : (a.man << (-sh));
    bool frac = sh > 0 && (a.man & ((((u128)1) << sh) - 1)) != 0;
    long long v = (long long)ip;
    if (a.sign) return -v - (frac ? 1 : 0);
    return v;
}

// to IEEE binary128 bit pattern (tests compare against __float128)
SMC_HD void q128_bits(q128 a, uint64_t &hi, uint64_t &lo) {
    if (a.man == 0) { hi = (uint64_t)a.sign << 63; lo = 0; return; }
    u128 frac = a.man & ((((u128)1) << 112) - 1);
    u128 bexp = (u128)(a.exp + 16383);
    u128 bits = ((u128)a.sign << 127) | (bexp << 112) | frac;
    hi = (uint64_t)(bits >> 64);
    lo = (uint64_t)bits;
}

}  // namespace smc
