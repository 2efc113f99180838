// Integer arithmetic shared by the sieve kernels and by the host-side unit
// tests (the same source compiles for sm_103a and for the CPU).
//
// Contents
//   * modular helpers for 32-bit and 64-bit primes (p < 2^46);
//   * Montgomery reduction used by the K mod p kernel;
//   * pg_modsearch*: smallest k >= 1 with l <= k*a mod p <= r, the problem
//     solved by _modulo_search_euclid / _modulo_search_euclid_stack
//     (modulo_search.cpp:71-193), here as an iterative descent with an
//     explicit stack whose unwinding also returns the residue k*a mod p;
//   * pg_three_gap: the two "record" multiples of a modulo p that decide every
//     return of the orbit y -> y + a (mod p) to the window [0, w) (Slater's
//     three-gap theorem), computed by a subtractive continued fraction;
//   * pg_hits_*: all mi in [mi_lo, mi_hi) with (r*(M+mi) + SL) mod p <= 2*SL,
//     i.e. the enumeration of modulo_search_euclid_all_large
//     (modulo_search.cpp:339-376), at O(1) per hit after one search.
#pragma once
#include <stdint.h>

#if !defined(__CUDA_ARCH__)
#include <math.h>
#endif

#if defined(__CUDACC__)
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pg {

PG_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// x mod p for p < 2^46 and x < 2^64, from a double-precision quotient
// estimate corrected with exact 64-bit wrap-around arithmetic.
PG_HD uint64_t mod_u64(uint64_t x, uint64_t p, double inv_p) {
    uint64_t q = (uint64_t)((double)x * inv_p);
    int64_t r = (int64_t)(x - q * p);
    while (r < 0) r += (int64_t)p;
    while (r >= (int64_t)p) r -= (int64_t)p;
    return (uint64_t)r;
}

// a*b mod p for a, b < p < 2^46 (the product fits in 92 bits; the quotient
// estimate a*b/p < 2^46 is within 1 of the truth).
PG_HD uint64_t mulmod_u64(uint64_t a, uint64_t b, uint64_t p, double inv_p) {
    uint64_t q = (uint64_t)((double)a * (double)b * inv_p);
    int64_t r = (int64_t)(a * b - q * p);
    while (r < 0) r += (int64_t)p;
    while (r >= (int64_t)p) r -= (int64_t)p;
    return (uint64_t)r;
}

// -p^{-1} mod 2^32 for odd p (Newton iteration on the 2-adic inverse).
PG_HD uint32_t neg_inv32(uint32_t p) {
    uint32_t x = (3u * p) ^ 2u;  // correct to 5 bits
    for (int i = 0; i < 3; i++) x *= 2u - p * x;
    return 0u - x;
}

// -p^{-1} mod 2^64 for odd p: the 32-bit inverse (three 32-bit steps from
// 5 bits), then one 64-bit Newton step doubles it to 64 bits.
PG_HD uint64_t neg_inv64(uint64_t p) {
    const uint32_t p32 = (uint32_t)p;
    uint32_t x32 = (3u * p32) ^ 2u;
    for (int i = 0; i < 3; i++) x32 *= 2u - p32 * x32;
    uint64_t x = x32;
    x *= 2ull - p * x;
    return 0ull - x;
}

// Montgomery reduction, R = 2^32: t * 2^-32 mod p (result < 2p) for t < p*2^32.
// For p < 2^31 and t < 2p^2 + 2^32 the sum t + m*p stays below 2^64, so it
// is one multiply-add whose high word is the result.
PG_HD uint32_t redc32_lazy(uint64_t t, uint32_t p, uint32_t pinv) {
    const uint32_t m = (uint32_t)t * pinv;
    return (uint32_t)((t + (uint64_t)m * p) >> 32);
}

PG_HD uint32_t umulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// ---------------------------------------------------------------------------
// two 32-bit quotients by one divisor
//
// Division by multiplication with an approximate reciprocal and a remainder
// correction (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994).  r = floor(x), x = 2^32 (1 - 2^-19) / d in
// single precision: a reciprocal of at most 1 ulp error (rcp.approx) of d
// rounded toward zero, times 2^32 - 2^13 rounded toward zero.  Then
//   2^32/d (1 - 2^-18) - 1 <= r < 2^32/d,
// so q0 = floor(n r / 2^32) never exceeds q = floor(n / d), and while
// q < 2^18 it is at most 2 below it (n/d - n r/2^32 < (n/d) 2^-18 + 1 < 2);
// q0 < 2^17 implies q < 2^18.  Two remainder tests per quotient finish it;
// a larger q0 (a continued-fraction quotient of 2^17 or more, rare) takes
// the exact division.  One reciprocal (three conversion/transcendental-unit
// operations) serves both quotients, where two hardware divisions each
// need their own.

// single-precision steps with explicit rounding; the host forms compute the
// same roundings exactly (the reciprocal within the device's 1-ulp bound)
PG_HD float u32_to_f32_rz(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __uint2float_rz(v);
#else
    float f = (float)v;
    if ((double)f > (double)v) f = nextafterf(f, 0.0f);
    return f;
#endif
}
// v rounded toward zero to 24 bits (exact top-24-bit truncation).
PG_HD float u64_trunc24(uint64_t v) {
#if defined(__CUDA_ARCH__)
    const int sh = v < (1ull << 24) ? 0 : 64 - __clzll((long long)v) - 24;
#else
    const int sh = v < (1ull << 24) ? 0 : 64 - __builtin_clzll(v) - 24;
#endif
    return ldexpf((float)(v >> sh), sh);
}
// A 64-bit value in single precision rounded toward zero through its two
// 32-bit halves: rz(rz(hi) 2^32 + rz(lo)), at most 2^-22 below v and never
// above it.  (A direct 64-bit conversion runs on the double-precision pipe,
// which is narrow on this part.)
PG_HD float u64_to_f32_rz(uint64_t v) {
    const uint32_t hi = (uint32_t)(v >> 32), lo = (uint32_t)v;
#if defined(__CUDA_ARCH__)
    if (hi == 0) return __uint2float_rz(lo);
    return __fadd_rz(__fmul_rz(__uint2float_rz(hi), 4294967296.0f), __uint2float_rz(lo));
#else
    if (hi == 0) return u32_to_f32_rz(lo);
    // the exact sum of the two rounded halves, then rounded toward zero
    const uint64_t s = ((uint64_t)u32_to_f32_rz(hi) << 32) + (uint64_t)u32_to_f32_rz(lo);
    return u64_trunc24(s);
#endif
}
PG_HD float as_f32(uint32_t v) { return (float)v; }
PG_HD float as_f32(uint64_t v) { return u64_to_f32_rz(v); }
PG_HD float rcp_approx(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
PG_HD float mul_f32_rz(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rz(a, b);
#else
    const double e = (double)a * (double)b;  // exact: 24 + 24 bits
    float f = (float)e;
    if ((double)f > e) f = nextafterf(f, 0.0f);
    return f;
#endif
}
PG_HD uint32_t f32_to_u32_rz(float x) {
#if defined(__CUDA_ARCH__)
    return __float2uint_rz(x);
#else
    return x >= 4294967296.0f ? 0xFFFFFFFFu : (uint32_t)x;  // saturates as the device does
#endif
}

// r of the comment above for d >= 1.  `skew` (host tests only) moves the
// reciprocal by that many ulps to cover the device's error bound.
PG_HD uint32_t recip32(uint32_t d, int skew = 0) {
    float rf = rcp_approx(u32_to_f32_rz(d));
#if !defined(__CUDA_ARCH__)
    for (; skew > 0; skew--) rf = nextafterf(rf, 2.0f);
    for (; skew < 0; skew++) rf = nextafterf(rf, 0.0f);
#else
    (void)skew;
#endif
    return f32_to_u32_rz(mul_f32_rz(rf, 4294959104.0f));  // 2^32 - 2^13
}

PG_HD void udiv2_32(uint32_t n1, uint32_t n2, uint32_t d, uint32_t &q1, uint32_t &q2, int skew = 0) {
    const uint32_t r = recip32(d, skew);
    uint32_t a = umulhi32(n1, r), b = umulhi32(n2, r);
    if ((a | b) >= (1u << 17)) {
        q1 = n1 / d;
        q2 = n2 / d;
        return;
    }
    uint32_t ra = n1 - a * d, rb = n2 - b * d;
    if (ra >= d) a++, ra -= d;
    if (ra >= d) a++;
    if (rb >= d) b++, rb -= d;
    if (rb >= d) b++;
    q1 = a;
    q2 = b;
}

// Two 32-bit quotients by one divisor with the quotients themselves taken in
// single precision (the bound of udiv2_64 below): one remainder test each
// instead of two, for two more conversions.
PG_HD void udiv2f_32(uint32_t n1, uint32_t n2, uint32_t d, uint32_t &q1, uint32_t &q2, int skew = 0) {
    float rf = rcp_approx(u32_to_f32_rz(d));
#if !defined(__CUDA_ARCH__)
    for (; skew > 0; skew--) rf = nextafterf(rf, 2.0f);
    for (; skew < 0; skew++) rf = nextafterf(rf, 0.0f);
#else
    (void)skew;
#endif
    const float rs = mul_f32_rz(rf, 0.999998092651367188f);  // 1 - 2^-19
    const uint32_t a = f32_to_u32_rz(mul_f32_rz(u32_to_f32_rz(n1), rs));
    const uint32_t b = f32_to_u32_rz(mul_f32_rz(u32_to_f32_rz(n2), rs));
    if ((a | b) >= (1u << 17)) {
        q1 = n1 / d;
        q2 = n2 / d;
        return;
    }
    q1 = a + (n1 - a * d >= d ? 1u : 0u);
    q2 = b + (n2 - b * d >= d ? 1u : 0u);
}

// Two 64-bit quotients by one divisor, the same way in single precision:
// x = (n_f * rs) with n_f = n rounded toward zero (u64_to_f32_rz: within
// 2^-22), rs = rcp(d_f) (1 - 2^-19) rounded toward zero, d_f = d rounded
// toward zero.  With the reciprocal within 3 ulps, (n/d)(1 - 2^-18) < x <
// n/d, so q0 = floor(x)
// never exceeds q = floor(n/d) and, while q0 < 2^17 (hence n/d < 2^18), is
// at least q - 1: one remainder test finishes it.  A larger q0 takes the
// exact division.
PG_HD void udiv2_64(uint64_t n1, uint64_t n2, uint64_t d, uint64_t &q1, uint64_t &q2, int skew = 0) {
    float rf = rcp_approx(u64_to_f32_rz(d));
#if !defined(__CUDA_ARCH__)
    for (; skew > 0; skew--) rf = nextafterf(rf, 2.0f);
    for (; skew < 0; skew++) rf = nextafterf(rf, 0.0f);
#else
    (void)skew;
#endif
    const float rs = mul_f32_rz(rf, 0.999998092651367188f);  // 1 - 2^-19, exact in single precision
    const uint32_t a = f32_to_u32_rz(mul_f32_rz(u64_to_f32_rz(n1), rs));
    const uint32_t b = f32_to_u32_rz(mul_f32_rz(u64_to_f32_rz(n2), rs));
    if ((a | b) >= (1u << 17)) {
        q1 = n1 / d;
        q2 = n2 / d;
        return;
    }
    const uint64_t ra = n1 - (uint64_t)a * d, rb = n2 - (uint64_t)b * d;
    q1 = a + (ra >= d ? 1u : 0u);
    q2 = b + (rb >= d ? 1u : 0u);
}

// 2^64 mod p and 2^128 mod p for odd 3 <= p < 2^46 with neither a division
// nor double precision: x <- x 2^16 mod p eight times from x = 1.  Each
// step's quotient is below 2^16 (x < p), so one single-precision reciprocal
// gives it or one less (the bound of udiv2_64) and one remainder test ends it.
PG_HD void pow64_128_mod(uint64_t p, uint64_t &r1, uint64_t &r2, int skew = 0) {
    float rf = rcp_approx(u64_to_f32_rz(p));
#if !defined(__CUDA_ARCH__)
    for (; skew > 0; skew--) rf = nextafterf(rf, 2.0f);
    for (; skew < 0; skew++) rf = nextafterf(rf, 0.0f);
#else
    (void)skew;
#endif
    const float rs = mul_f32_rz(rf, 0.999998092651367188f);  // 1 - 2^-19
    uint64_t x = 1;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint64_t n = x << 16;  // < 2^62
        const uint32_t q = f32_to_u32_rz(mul_f32_rz(u64_to_f32_rz(n), rs));
        uint64_t t = n - (uint64_t)q * p;
        x = t >= p ? t - p : t;
        if (i == 3) r1 = x;
    }
    r2 = x;
}

// 2^32 mod p for odd p >= 3 without a hardware division.  p >= 2^31: 2^32 - p.
// 2^16 <= p < 2^31: q0 = recip32(p) is at most floor(2^32/p) and at most one
// below it ((2^32/p) 2^-18 + 1 < 2), so 2^32 - q0 p lies in [0, 3p) and two
// conditional subtractions finish it.  Smaller p: the remainder operator.
PG_HD uint32_t pow32_mod(uint32_t p, int skew = 0) {
    if (p >= 0x80000000u) return 0u - p;
    if (p < (1u << 16)) return (0u - p) % p;
    uint32_t r = 0u - recip32(p, skew) * p;
    r = r >= p ? r - p : r;
    return r >= p ? r - p : r;
}

PG_HD uint32_t redc32(uint64_t t, uint32_t p, uint32_t pinv) {
    const uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
    const uint32_t m = lo * pinv;
    // hi < p and hi(m*p) < p, so the true sum is below 2p < 2^33: at most
    // one wrap, which shows as s < a
    const uint32_t a = hi + (lo != 0u);
    const uint32_t s = a + umulhi32(m, p);
    return (s < a || s >= p) ? s - p : s;
}

// R^2 mod p (R = 2^32) from r1 = R mod p without a 64-bit division: x = 2^33
// mod p (one doubling), then five Montgomery squarings, each sending the
// power e of x = 2^e to 2e - 32: 33 -> 34 -> 36 -> 40 -> 48 -> 64.
PG_HD uint32_t r2_from_r1(uint32_t r1, uint32_t p, uint32_t pinv) {
    uint32_t x = r1 >= p - r1 ? r1 - (p - r1) : r1 + r1;
    for (int i = 0; i < 5; i++) x = redc32((uint64_t)x * x, p, pinv);
    return x;
}

// Montgomery reduction, R = 2^64, of the 128-bit value (hi:lo) < p*2^64;
// p < 2^63.  Result in [0, p).
PG_HD uint64_t redc64(uint64_t hi, uint64_t lo, uint64_t p, uint64_t pinv) {
    uint64_t m = lo * pinv;
    uint64_t s_hi = umulhi64(m, p);
    // lo + m*p_lo == 0 mod 2^64, carry out iff lo != 0
    uint64_t r = hi + s_hi + (lo != 0);
    return r >= p ? r - p : r;
}

// ---------------------------------------------------------------------------
// K mod p by Montgomery multiplication over the limbs of K, most significant
// first: u <- REDC(u * R^2 + limb) gives u = K * R^-1 after the last limb, and
// REDC(u * R^2) = K mod p.

// 32-bit odd primes; lazy reduction keeps u < 2p while p < 2^31.
PG_HD uint32_t kmod32(const uint32_t *limbs, int n, uint32_t p, uint32_t &pinv_out,
                      uint32_t &r2_out) {
    const uint32_t pinv = neg_inv32(p);
    const uint32_t r1 = (0u - p) % p;                          // 2^32 mod p
    const uint32_t r2 = r2_from_r1(r1, p, pinv);               // 2^64 mod p
    uint32_t u = 0;
    if (p < 0x80000000u) {
        for (int i = n - 1; i >= 0; i--) u = redc32_lazy((uint64_t)u * r2 + limbs[i], p, pinv);
        if (u >= p) u -= p;
    } else {
        for (int i = n - 1; i >= 0; i--) u = redc32((uint64_t)u * r2 + limbs[i], p, pinv);
    }
    pinv_out = pinv;
    r2_out = r2;
    return redc32((uint64_t)u * r2, p, pinv);
}

// kmod32 for NP primes at once: NP independent Montgomery chains share each
// limb read and hide each other's multiply latency.
template <int NP>
PG_HD void kmod32_multi(const uint32_t *limbs, int n, const uint32_t *p, uint32_t *r,
                        uint32_t *pinv, uint32_t *r2) {
    uint32_t u[NP];
    bool lazy = true;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        pinv[k] = neg_inv32(p[k]);
        const uint32_t r1 = pow32_mod(p[k]);
        r2[k] = r2_from_r1(r1, p[k], pinv[k]);
        u[k] = 0;
        lazy = lazy && p[k] < 0x80000000u;
    }
    if (lazy) {
        for (int i = n - 1; i >= 0; i--) {
            const uint32_t l = limbs[i];
#pragma unroll
            for (int k = 0; k < NP; k++) u[k] = redc32_lazy((uint64_t)u[k] * r2[k] + l, p[k], pinv[k]);
        }
#pragma unroll
        for (int k = 0; k < NP; k++)
            if (u[k] >= p[k]) u[k] -= p[k];
    } else {
        for (int i = n - 1; i >= 0; i--) {
            const uint32_t l = limbs[i];
#pragma unroll
            for (int k = 0; k < NP; k++) u[k] = redc32((uint64_t)u[k] * r2[k] + l, p[k], pinv[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < NP; k++) r[k] = redc32((uint64_t)u[k] * r2[k], p[k], pinv[k]);
}

// (r * M + sl) mod p with the Montgomery constants of p (M < 3 * 2^32, sl < p).
PG_HD uint32_t start32(uint32_t r, uint64_t M, uint32_t sl, uint32_t p, uint32_t pinv,
                       uint32_t r2) {
    if ((M >> 32) == 0) {
        // M * r2 < 2^32 p: REDC(M r2) = M R mod p, and REDC(r M R) = r M mod p
        const uint32_t mr = redc32(M * r2, p, pinv);
        const uint32_t rm = redc32((uint64_t)r * mr, p, pinv);
        const uint64_t t = (uint64_t)rm + sl;
        return (uint32_t)(t >= p ? t - p : t);
    }
    uint32_t a = redc32(M, p, pinv);                  // M R^-1
    uint32_t mm = redc32((uint64_t)a * r2, p, pinv);  // M mod p
    uint32_t b = redc32((uint64_t)r * mm, p, pinv);   // r M R^-1
    uint32_t rm = redc32((uint64_t)b * r2, p, pinv);  // r M mod p
    uint64_t t = (uint64_t)rm + sl;
    return (uint32_t)(t >= p ? t - p : t);
}

// ---------------------------------------------------------------------------
// K mod p, least significant limb first: W <- REDC(W + limb) leaves
// W = K * R^-n after n limbs (each step multiplies what came before by R^-1),
// and REDC(W * R^(n+1)) = K mod p.  A step is one add and one REDC (two
// multiplies) instead of the most-significant-first step's three; R^(n+1) mod p
// costs log2(n) Montgomery squarings and popcount(n) - 1 products per prime,
// outweighed by the cheaper steps for long K.

// (W + l) * 2^-32 mod p, result <= p + 1, for W <= p + 1, p < 2^32 - 4.
// x + m*p <= (p + 2^32) + (2^32 - 1)p = 2^32 (p + 1) < 2^64: one multiply-add.
PG_HD uint32_t redc32_add(uint32_t W, uint32_t l, uint32_t p, uint32_t pinv) {
    const uint64_t x = (uint64_t)W + l;  // < 2^33
    const uint32_t m = (uint32_t)x * pinv;
    return (uint32_t)((x + (uint64_t)m * p) >> 32);
}

// NP primes (odd, 3 <= p < 2^32 - 4) at once, least significant limb first
// (n >= 1 limbs).  Also returns pinv and r2 = 2^64 mod p of each prime.
template <int NP>
PG_HD void kmod32_lsb_multi(const uint32_t *limbs, int n, const uint32_t *p, uint32_t *r,
                            uint32_t *pinv, uint32_t *r2) {
    uint32_t W[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) {
        pinv[k] = neg_inv32(p[k]);
        r2[k] = r2_from_r1(pow32_mod(p[k]), p[k], pinv[k]);
        W[k] = 0;
    }
#pragma unroll 4
    for (int i = 0; i < n; i++) {
        const uint32_t l = limbs[i];
#pragma unroll
        for (int k = 0; k < NP; k++) W[k] = redc32_add(W[k], l, p[k], pinv[k]);
    }
    // R^(n+1) mod p from r2 = R^2: with x = R^(f+1), a Montgomery square
    // gives R^(2f+1) and a product with r2 gives R^(f+2); the bits of n
    // after the leading one double f and add one (f = 1 to f = n)
    uint32_t X[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) X[k] = r2[k];
#if defined(__CUDA_ARCH__)
    const int top = 31 - __clz(n);  // n >= 1: the leading bit
#else
    const int top = 31 - __builtin_clz((unsigned)n);
#endif
    for (int b = top - 1; b >= 0; b--) {
        const bool one = ((uint32_t)n >> b) & 1u;
#pragma unroll
        for (int k = 0; k < NP; k++) {
            X[k] = redc32((uint64_t)X[k] * X[k], p[k], pinv[k]);
            if (one) X[k] = redc32((uint64_t)X[k] * r2[k], p[k], pinv[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < NP; k++)
        r[k] = redc32((uint64_t)W[k] * X[k], p[k], pinv[k]);  // W * X < (p + 2) * p < p * 2^32
}

// Odd primes 2^31 <= p < 2^46 (and any odd p >= 3 below that): R = 2^64.
PG_HD uint64_t kmod64(const uint32_t *limbs, int n, uint64_t p, uint64_t *pinv_out = nullptr,
                      uint64_t *r2_out = nullptr) {
    const uint64_t pinv = neg_inv64(p);
    uint64_t r1, r2;  // 2^64 and 2^128 mod p
    pow64_128_mod(p, r1, r2);
    if (pinv_out) *pinv_out = pinv, *r2_out = r2;
    uint64_t u = 0;
    const int nw = (n + 1) / 2;
    for (int i = nw - 1; i >= 0; i--) {
        uint64_t w = limbs[2 * i];
        if (2 * i + 1 < n) w |= (uint64_t)limbs[2 * i + 1] << 32;
        uint64_t lo = u * r2;
        uint64_t hi = umulhi64(u, r2);
        uint64_t lo2 = lo + w;
        hi += lo2 < lo;
        u = redc64(hi, lo2, p, pinv);
    }
    return redc64(umulhi64(u, r2), u * r2, p, pinv);
}

// REDC of the 65-bit value c*2^64 + lo (R = 2^64), result < p + 2 for
// c*2^64 + lo < 2^64 + p*2^64.
PG_HD uint64_t redc64_add(uint64_t W, uint64_t w, uint64_t p, uint64_t pinv) {
    const uint64_t lo = W + w;
    const uint64_t c = lo < W;
    const uint64_t m = lo * pinv;
    return c + umulhi64(m, p) + (lo != 0);
}

// Montgomery product for R = 2^64, inputs < p < 2^63, result < p.
PG_HD uint64_t montmul64(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv) {
    return redc64(umulhi64(a, b), a * b, p, pinv);
}

// kmod64 least significant 64-bit word first: W <- REDC(W + word), then
// K mod p = REDC(W * R^(nw+1)).  Odd p < 2^46.
PG_HD uint64_t kmod64_lsb(const uint32_t *limbs, int n, uint64_t p, uint64_t *pinv_out = nullptr,
                          uint64_t *r2_out = nullptr) {
    const uint64_t pinv = neg_inv64(p);
    uint64_t r1, r2;  // 2^64 and 2^128 mod p
    pow64_128_mod(p, r1, r2);
    if (pinv_out) *pinv_out = pinv, *r2_out = r2;
    const int nw = (n + 1) / 2;
    uint64_t W = 0;
    for (int i = 0; i < nw; i++) {
        uint64_t w = limbs[2 * i];
        if (2 * i + 1 < n) w |= (uint64_t)limbs[2 * i + 1] << 32;
        W = redc64_add(W, w, p, pinv);
    }
    uint64_t acc = r1, b = r2;
    for (uint32_t e = (uint32_t)nw; e;) {
        if (e & 1u) acc = montmul64(acc, b, p, pinv);
        e >>= 1;
        if (e) b = montmul64(b, b, p, pinv);
    }
    if (W >= p) W -= p;  // W < p + 2
    return montmul64(W, acc, p, pinv);
}

// ---------------------------------------------------------------------------
// modulo search
//
// Smallest k >= 1 with l <= (k*a mod p) <= r, for 0 < a < p, 1 <= l <= r < p.
// Follows the reduction of modulo_search.cpp:131-193: mirror when a > p/2,
// answer directly when a multiple of a falls in [l, r], otherwise recurse on
// (a, a - p mod a, l mod a, r mod a).  Also returns the residue k*a mod p.
//
// Unwinding uses k_i = (k_{i+1} p_i + v_{i+1}) / a_i + floor((l_i - 1)/a_i),
// an exact division, where v is the residue of the deeper level; the residue
// of each level is v_i = floor((l_i-1)/a_i)*a_i + v_{i+1} (no reduction
// needed since it lies in [l_i, r_i]), then un-mirrored.

struct ModSearch32 {
    uint32_t k;  // smallest k >= 1
    uint32_t v;  // k*a mod p, in [l, r]
};

// 32-bit primes: every level has p_i < 2^32, depth <= 32 (p halves per level).
PG_HD ModSearch32 modsearch32(uint32_t p, uint32_t a, uint32_t l, uint32_t r) {
    uint32_t st_p[32], st_a[32], st_ldiv[32];
    uint8_t st_mirror[32];
    int depth = 0;
    const uint32_t delta = r - l;
    uint32_t k, v;
    for (;;) {
        bool mirror = a > (p >> 1);
        if (mirror) {
            // k*a in [l, r]  <=>  k*(p-a) in [p-r, p-l]
            a = p - a;
            l = p - (l + delta);
        }
        uint32_t l_div = (l - 1) / a;
        uint32_t l_mod = l - l_div * a;  // in [1, a]
        if (l_mod + delta >= a) {
            // (l_div + 1) * a lies in [l, r]
            k = l_div + 1;
            v = k * a;
            if (mirror) v = p - v;
            break;
        }
        if (depth >= 31) {
            // unreachable for 0 < a < p < 2^32 (p halves per level); bail out
            // with "no solution below p" rather than overflow the stack
            k = 0xFFFFFFFFu;
            v = l;
            depth = 0;
            break;
        }
        st_p[depth] = p;
        st_a[depth] = a;
        st_ldiv[depth] = l_div;
        st_mirror[depth] = mirror;
        depth++;
        uint32_t new_a = a - (p % a);
        p = a;
        a = new_a;
        l = l_mod;
    }
    while (depth > 0) {
        depth--;
        uint32_t pi = st_p[depth], ai = st_a[depth], ldiv = st_ldiv[depth];
        // v is the pre-mirror residue of the deeper level: k*(a_i - p_i mod a_i) mod a_i
        uint64_t num = (uint64_t)k * pi + v;
        uint32_t q = (uint32_t)(num / ai);
        k = q + ldiv;
        v = ldiv * ai + v;  // post-mirror residue at this level, in [l_i, r_i]
        if (st_mirror[depth]) v = pi - v;
    }
    return {k, v};
}

struct ModSearch64 {
    uint64_t k;
    uint64_t v;
};

// Primes up to 2^46.  Levels whose modulus is below 2^32 continue in 32-bit.
PG_HD ModSearch64 modsearch64(uint64_t p, uint64_t a, uint64_t l, uint64_t r) {
    if (p < 0xFFFFFFFFull) {
        ModSearch32 s = modsearch32((uint32_t)p, (uint32_t)a, (uint32_t)l, (uint32_t)r);
        return {s.k, s.v};
    }
    uint64_t st_p[24], st_a[24], st_ldiv[24];
    uint8_t st_mirror[24];
    int depth = 0;
    const uint64_t delta = r - l;
    uint64_t k, v;
    for (;;) {
        if (p < 0xFFFFFFFFull) {
            ModSearch32 s = modsearch32((uint32_t)p, (uint32_t)a, (uint32_t)l,
                                        (uint32_t)(l + delta));
            k = s.k;
            v = s.v;
            break;
        }
        bool mirror = a > (p >> 1);
        if (mirror) {
            a = p - a;
            l = p - (l + delta);
        }
        uint64_t l_div = (l - 1) / a;
        uint64_t l_mod = l - l_div * a;
        if (l_mod + delta >= a) {
            k = l_div + 1;
            v = k * a;
            if (mirror) v = p - v;
            break;
        }
        if (depth >= 23) {
            k = ~0ull >> 1;  // unreachable for p < 2^46; see modsearch32
            v = l;
            depth = 0;
            break;
        }
        st_p[depth] = p;
        st_a[depth] = a;
        st_ldiv[depth] = l_div;
        st_mirror[depth] = mirror;
        depth++;
        uint64_t new_a = a - (p % a);
        p = a;
        a = new_a;
        l = l_mod;
    }
    while (depth > 0) {
        depth--;
        uint64_t pi = st_p[depth], ai = st_a[depth], ldiv = st_ldiv[depth];
        // num = k*p_i + v < 2^(46+46); quotient < p_i < 2^46
        uint64_t lo = k * pi;
        uint64_t hi = umulhi64(k, pi);
        uint64_t lo2 = lo + v;
        hi += (lo2 < lo);
        // exact division of (hi:lo2) by ai with quotient < 2^46
        double est = ((double)hi * 18446744073709551616.0 + (double)lo2) / (double)ai;
        uint64_t q = (uint64_t)est;
        // correct: rem = num - q*ai in signed 64-bit (|rem| small)
        int64_t rem = (int64_t)(lo2 - q * ai);
        while (rem < 0) {
            q--;
            rem += (int64_t)ai;
        }
        while (rem >= (int64_t)ai) {
            q++;
            rem -= (int64_t)ai;
        }
        k = q + ldiv;
        v = ldiv * ai + v;
        if (st_mirror[depth]) v = pi - v;
    }
    return {k, v};
}

// ---------------------------------------------------------------------------
// three-gap structure of the rotation y -> y + a (mod p) on the window [0, w)
//
// kp = smallest k >= 1 with (k*a mod p) in (0, w),      up  = that residue
// kn = smallest k >= 1 with (-(k*a) mod p) in (0, w),   dn  = that residue
// For p > 2w, the first return time from y in [0, w) is
//   kp       if y + up < w           (landing at y + up)
//   kn       else if y >= dn         (landing at y - dn)
//   kp + kn  otherwise               (landing at y + up - dn).
// (up + dn >= w always holds, so the first two cases are exclusive.)
// Computed by the subtractive continued fraction that keeps the lattice basis
// (kp, up), (kn, -dn) with kp*dn + kn*up = p, reducing the larger residue by
// the smaller until both are below w.
template <typename T>
struct ThreeGap {
    T kp, up, kn, dn;
};

template <typename T>
PG_HD ThreeGap<T> three_gap(T p, T a, T w) {
    T kp = 1, up = a, kn = 1, dn = p - a;
    // Each pass lowers up or dn by at least one; the pass limit only guards
    // against non-prime moduli (for prime p, up == dn forces up == dn == 1).
    for (int pass = 0; pass < 256 && (up >= w || dn >= w); pass++) {
        if (up > dn) {
            T q1 = (up - w) / dn + 1;  // first multiple that brings up below w
            T q2 = (up - 1) / dn;      // multiples that keep up > 0 and stop at up <= dn
            T q = q1 < q2 ? q1 : q2;
            if (q == 0) break;
            up -= q * dn;
            kp += q * kn;
        } else {
            T q1 = (dn - w) / up + 1;
            T q2 = (dn - 1) / up;
            T q = q1 < q2 ? q1 : q2;
            if (q == 0) break;
            dn -= q * up;
            kn += q * kp;
        }
    }
    return {kp, up, kn, dn};
}

// ---------------------------------------------------------------------------
// parity-reduced walk of a large prime
//
// Only odd m*K + X can be prime.  For d even, valid m are odd and K is odd,
// so X must be even: with m = m0 + 2j and X = 2X', p | m*K + X becomes
// X' == -m*K/2 (mod p), a walk in j whose step is r = K mod p again
// (2 * (1/2) = 1), over a window of 2*floor(SL/2)+1 values of X'.  For d odd,
// K is even and X must be odd: X = 2X' + 1 gives X' == -(m*K + 1)/2, a walk
// in m with step r/2 mod p.  Either way the residue of walk index 0 is
// t0 = (r/2 * m0 + c) mod p, with c = floor(SL/2) (d even) or
// floor((SL-1)/2) + (p+1)/2 (d odd), and a residue Y < w is the hit
// X = xc - 2*Y - SL.  This removes the hits on even m*K + X before they are
// generated: 4x fewer walk steps for d even, 2x for d odd.
struct WalkParams {
    uint32_t stride;   // mi = mi_base + stride * j
    uint32_t mi_base;
    uint64_t jmax;     // walk indices j in [0, jmax)
    uint32_t w;        // hits: residue Y < w
    uint32_t xc;       // offset index x = X + SL = xc - 2*Y
    uint32_t c_add;    // floor(SL/2) (d even) or floor((SL-1)/2) (d odd)
    uint32_t odd_d;    // 1 when d is odd: step r/2, constant c_add + (p+1)/2
    uint64_t m0;       // m of walk index 0
};

// r / 2 mod p for odd p.
PG_HD uint32_t half_mod(uint32_t r, uint32_t p) {
    return (r & 1u) ? (uint32_t)(((uint64_t)r + p) >> 1) : (r >> 1);
}
PG_HD uint64_t half_mod(uint64_t r, uint64_t p) { return (r & 1u) ? ((r + p) >> 1) : (r >> 1); }

// Step and start residue of a prime's parity-reduced walk from r = K mod p:
// step = r/2 (d odd) or r (d even); t0 = (step' * m0 + c) mod p with
// step' = r/2 and c = c_add (+ (p+1)/2 when d is odd).  r2 = 2^64 mod p
// (32-bit primes only; it comes with K mod p).
// kmul != 1: r is K' mod p for K = K' * kmul; K mod p = REDC(REDC(r * kmul) * r2).
// pinv: -p^-1 mod 2^32 when the caller has it, else 0 (computed here).
PG_HD void walk_start(const WalkParams &wk, uint32_t p, uint32_t r, uint32_t r2, uint32_t &step,
                      uint32_t &t0, uint32_t kmul = 1, uint32_t pinv = 0) {
    if (pinv == 0) pinv = neg_inv32(p);
    if (kmul != 1) r = redc32((uint64_t)redc32((uint64_t)r * kmul, p, pinv) * r2, p, pinv);
    const uint32_t rh = half_mod(r, p);
    const uint32_t c = wk.c_add + (wk.odd_d ? (p >> 1) + 1 : 0u);
    step = wk.odd_d ? rh : r;
    t0 = start32(rh, wk.m0, c, p, pinv, r2);
}
// 64-bit primes (p < 2^46, any m0): with pinv = -p^-1 mod 2^64 and
// r2 = 2^128 mod p, t0 = REDC(REDC(m0 * r2) * rh) + c = m0 * rh + c mod p,
// with no division.
PG_HD void walk_start(const WalkParams &wk, uint64_t p, uint64_t r, uint64_t pinv, uint64_t r2,
                      uint64_t &step, uint64_t &t0, uint32_t kmul = 1) {
    if (kmul != 1) r = montmul64(montmul64(r, kmul, p, pinv), r2, p, pinv);
    const uint64_t rh = half_mod(r, p);
    const uint64_t c = wk.c_add + (wk.odd_d ? (p >> 1) + 1 : 0ull);
    const uint64_t m0R = montmul64(wk.m0, r2, p, pinv);  // m0 * 2^64 mod p
    uint64_t t = montmul64(m0R, rh, p, pinv) + c;
    if (t >= p) t -= p;
    step = wk.odd_d ? rh : r;
    t0 = t;
}


// ---------------------------------------------------------------------------
// first entry and three-gap data in one continued-fraction pass
//
// The subtractive continued fraction of three_gap is a Rauzy induction of the
// rotation y -> y + a (mod p): every level (kp, up, kn, dn) is itself a
// rotation by `up` on a circle of length C = up + dn, whose steps cost kp
// (no wrap) or kn (wrap) units of the original time, and which is the
// first-return map of the original rotation to [0, C).  Going one level down
// shrinks the circle to C' = max(up, dn), and a point of [0, C) enters
// [0, C') after at most one step (a wrap, y -> y - dn).  Following the start
// point y0 through every level therefore gives the first time t >= 0 with
// (y0 + t*a) mod p < w, and its residue, at O(1) per batch of levels -- no
// separate modulo search.  Requires p > 2w, 0 < a < p, y0 < p.
template <typename T>
struct Entry {
    uint64_t t;  // first k >= 0 with (y0 + k*a) mod p in [0, w)
    T y;         // that residue, < w
    ThreeGap<T> g;
};

// Levels alternate: a level with up > dn leaves up' <= max(w - 1, dn), so
// either up' <= dn (the next level has dn > up') or both gaps are below w and
// the descent ends (for a prime modulus up' == dn cannot happen above 1).  The
// loop therefore runs the two kinds of level in turn, each with its roles
// fixed in the code: no per-level selects, and every lane of a warp runs the
// same kind of level at the same time.  The first level must have up > dn:
// for a < p - a the search runs on the mirror image z = (w - 1 - y) mod p,
// which maps [0, w) onto itself and turns the rotation by a into the rotation
// by p - a; the answer maps back by y = w - 1 - z and the three-gap data by
// swapping (kp, up) with (kn, dn).
//
// One level with big > small (up > dn, or dn > up in the other kind): big
// loses q copies of small, with q the least count leaving big <= max(w - 1,
// small), i.e. q = floor(min(C - w, big - 1) / small) with C = up + dn, and
// its m-step gains q copies of the other's.  The entry point y in [0, C)
// moves as follows, with f = floor((C - 1 - y) / small) (ceil((big - y) /
// small) for y < big, 0 otherwise):
//   up > dn: sub-level i of the batch enters [0, up - i*dn): y -= dn whenever
//            y >= up - i*dn, which, once true, stays true: q - f subtractions;
//   dn > up: sub-level i enters [0, dn - i*up) with one wrap y -= dn - i*up
//            at the first i where y >= dn - i*up, i = f (after it y < up).
// Both quotients share the divisor and one approximate reciprocal.
//
// Time: t only grows, and the first hit comes no earlier than the first
// entry into the current circle, so once t >= t_lim the search stops (no hit
// below t_lim): the caller sees t >= t_lim.  The loop keeps the budget
// rem = lim - t in the modulus' width: each increment dt is at most p (it is
// at most the level's new kp or kn, and kp*dn + kn*up = p), and for 32-bit
// moduli the true first entry is below p < 2^32 - 1, so a limit above 2^32 - 1
// never triggers and clamping it there changes nothing.
template <typename T>
PG_HD void quot2(T n1, T n2, T d, T &q1, T &q2) {
    if constexpr (sizeof(T) == 4) {
        udiv2f_32(n1, n2, d, q1, q2);
    } else {
        udiv2_64(n1, n2, d, q1, q2);
    }
}

template <typename T>
PG_HD Entry<T> first_entry(T p, T a, T w, T y0, uint64_t t_lim = ~0ull) {
    const bool mir = a < p - a;
    T up = mir ? p - a : a, dn = p - up, kp = 1, kn = 1;
    T y = !mir ? y0 : (y0 < w ? w - 1 - y0 : p - (y0 - (w - 1)));
    const T lim = t_lim < (uint64_t)(T)~(T)0 ? (T)t_lim : (T)~(T)0;
    T rem = lim;
    // Every level with q >= 1 lowers its big gap by at least small >= 1, so
    // the loop ends; q == 0 only for a tie up == dn (not for a prime modulus).
    for (;;) {
        if (up < w) break;  // up > dn: both below w
        {
            const T C = up + dn, n1 = (C - w) < (up - 1) ? (C - w) : (up - 1);
            T q, f;
            quot2<T>(n1, C - 1 - y, dn, q, f);
            if (q == 0) break;
            if (f < q) {
                const T m = q - f, dt = m * kn;
                if (dt >= rem) return {(uint64_t)(lim - rem) + dt, y, {kp, up, kn, dn}};
                y -= m * dn;
                rem -= dt;
            }
            up -= q * dn;
            kp += q * kn;
        }
        if (dn < w) break;  // dn > up: both below w
        {
            const T C = up + dn, n1 = (C - w) < (dn - 1) ? (C - w) : (dn - 1);
            T q, f;
            quot2<T>(n1, C - 1 - y, up, q, f);
            if (q == 0) break;
            if (f < q) {
                const T dt = kn + f * kp;
                if (dt >= rem) return {(uint64_t)(lim - rem) + dt, y, {kp, up, kn, dn}};
                y -= dn - f * up;
                rem -= dt;
            }
            dn -= q * up;
            kn += q * kp;
        }
    }
    uint64_t t = lim - rem;
    if (y >= w) {  // last level: [0, up + dn) -> [0, w) by one wrap
        y -= dn;
        t += kn;
    }
    if (mir) return {t, w - 1 - y, {kn, dn, kp, up}};
    return {t, y, {kp, up, kn, dn}};
}

// Rotation form of the hits after the first one: step n from a hit
// (mi0, y0) lands at Y = y0 + n*up, residue Y mod C, and
// mi = mi0 + (n - W)*kp + W*kn with W = floor(Y / C); it is a hit iff the
// residue is below w.  Returns an upper bound on the steps n with mi < mi_hi
// (mi_n - mi0 >= n*p/C - kp - kn since kp*dn + kn*up = p).
// Also: every step advances mi by at least min(kp, kn), so there are at most
// (mi_hi - mi0) / min(kp, kn) + 1 steps.  Single precision with a relative
// margin (each term within 2^-21, the margin 1.0001) and 2 added: the bound
// only sizes work, but must not fall below the true count.  Walk indices are
// below 2^31, so the span converts from 32 bits; a 32-bit prime's gaps and
// step costs too, with no 64-bit conversion or division.
template <typename T>
PG_HD uint64_t rotation_steps_bound(uint64_t mi0, uint64_t mi_hi, const ThreeGap<T> &g, T p) {
    if (mi0 >= mi_hi) return 0;
    const float span = (float)(uint32_t)(mi_hi - mi0);
    const float C = as_f32(g.up) + as_f32(g.dn);
    const float n = (span + as_f32(g.kp) + as_f32(g.kn)) * C * rcp_approx(as_f32(p));
    const float c = span * rcp_approx(as_f32(g.kp < g.kn ? g.kp : g.kn));
    return f32_to_u32_rz((n < c ? n : c) * 1.0001f + 2.0f);
}

// The rotation's walk in 32-bit arithmetic, for walk indices below
// mi_hi < 2^31 (any prime: gap32 below clamps a 64-bit prime's step costs).
// A step costing mi_hi or more ends the walk whatever its exact cost, so kp
// and kn are clamped to mi_hi and mi stays below 2^32.
//
// rotation_at32: position of rotation step n0 from the first hit (mi0, y0):
// Y = y0 + n0*up, residue Y mod C, mi = mi0 + (n0 - W)*kp + W*kn with
// W = floor(Y / C), clamped to mi_hi.
PG_HD void rotation_at32(uint32_t mi0, uint32_t y0, const ThreeGap<uint32_t> &g, uint32_t n0,
                         uint32_t mi_hi, uint32_t &y, uint32_t &mi) {
    const uint32_t C = g.up + g.dn;
    const uint64_t Y = y0 + (uint64_t)n0 * g.up;
    uint64_t W;
    if (n0 < (1u << 19)) {
        // W = floor(Y / C) <= n0 + 1 < 2^19 + 1 (y0 < C, up < C): a
        // single-precision quotient (from 32-bit operands, Y = y0 + n0 up)
        // is within 2^-20 relative, so within one
        W = f32_to_u32_rz(((float)n0 * (float)g.up + (float)y0) * rcp_approx((float)C));
        const int64_t rem = (int64_t)(Y - W * C);
        if (rem < 0) W--;
        else if (rem >= (int64_t)C) W++;
    } else {
        W = Y / C;
    }
    y = (uint32_t)(Y - W * C);
    const uint64_t m = mi0 + (n0 - W) * (uint64_t)g.kp + W * (uint64_t)g.kn;
    mi = m < mi_hi ? (uint32_t)m : mi_hi;
}

// A rotation's three-gap data in 32 bits for walks below mi_hi < 2^31:
// up, dn < w < 2^31, and step costs clamped to mi_hi (a step costing mi_hi
// or more ends the walk, and rotation_at32 clamps mi to mi_hi).
template <typename T>
PG_HD ThreeGap<uint32_t> gap32(const ThreeGap<T> &g, uint32_t mi_hi) {
    return ThreeGap<uint32_t>{g.kp < mi_hi ? (uint32_t)g.kp : mi_hi, (uint32_t)g.up,
                              g.kn < mi_hi ? (uint32_t)g.kn : mi_hi, (uint32_t)g.dn};
}

// rotation_walk32: up to `steps` rotation steps from (mi, y) while
// mi < mi_hi, calling emit(mi, y, y < w) at every step.  A step wraps when
// y + up >= C, i.e. y >= dn.  The definition of a walk's steps; the kernels
// run return_walk32 below, which visits the same hits and skips the misses
// (the host tests check the two against each other).
template <typename Emit>
PG_HD void rotation_walk32(uint32_t mi, uint32_t y, const ThreeGap<uint32_t> &g, uint32_t w,
                           uint32_t mi_hi, uint32_t steps, Emit &emit) {
    const uint32_t up = g.up, dn = g.dn;
    const uint32_t kp = g.kp < mi_hi ? g.kp : mi_hi, kn = g.kn < mi_hi ? g.kn : mi_hi;
    for (uint32_t k = 0; k < steps && mi < mi_hi; k++) {
        emit(mi, y, y < w);
        const bool wrap = y >= dn;
        y = wrap ? y - dn : y + up;
        mi += wrap ? kn : kp;
    }
}

// return_walk32: the same walk (the circle steps [0, steps) from (mi, y),
// while mi < mi_hi), visiting only its hits: from a hit y < w the next one
// is y + up (one step, kp) if that is below w, else y - dn (one step, kn) if
// y >= dn, else y + up - dn (two steps, the first off the window, kp + kn):
// the three-gap first-return map (p > 2w).  A start off the window (y >= w
// > dn) wraps into it in one step.  emit(mi, y, true) at every hit; about a
// third of a rotation's steps are misses, whose mask reads this saves.
// Step costs are clamped to mi_hi, so mi stays below 2 mi_hi < 2^32.
template <typename Emit>
PG_HD void return_walk32(uint32_t mi, uint32_t y, const ThreeGap<uint32_t> &g, uint32_t w, uint32_t mi_hi,
                         uint32_t steps, Emit &emit) {
    const uint32_t up = g.up, dn = g.dn;
    const uint32_t kp = g.kp < mi_hi ? g.kp : mi_hi, kn = g.kn < mi_hi ? g.kn : mi_hi;
    const uint32_t kpn = kp + kn < mi_hi ? kp + kn : mi_hi;
    uint32_t k = 0;
    if (y >= w && steps) {
        y -= dn;
        mi += kn;
        k = 1;
    }
    while (k < steps && mi < mi_hi) {
        emit(mi, y, true);
        const uint32_t a = y + up;
        const bool near = a < w, wrap = y >= dn;
        y = near ? a : (wrap ? y - dn : a - dn);
        mi += near ? kp : (wrap ? kn : kpn);
        k += (near | wrap) ? 1u : 2u;
    }
}

// ---------------------------------------------------------------------------
// hit enumeration

PG_HD void modsearch_any(uint32_t p, uint32_t a, uint32_t l, uint32_t r, uint64_t &k, uint32_t &v) {
    ModSearch32 s = modsearch32(p, a, l, r);
    k = s.k;
    v = s.v;
}
PG_HD void modsearch_any(uint64_t p, uint64_t a, uint64_t l, uint64_t r, uint64_t &k, uint64_t &v) {
    ModSearch64 s = modsearch64(p, a, l, r);
    k = s.k;
    v = s.v;
}

// y(mi_lo) = (t0 + mi_lo * r) mod p from y(0) = t0.
PG_HD uint32_t advance_residue(uint32_t t0, uint64_t mi_lo, uint32_t r, uint32_t p) {
    if (mi_lo == 0) return t0;
    uint32_t m = (uint32_t)(mi_lo % p);
    uint32_t s = (uint32_t)(((uint64_t)m * r) % p);
    uint32_t y = t0 + s;
    if (y >= p || y < t0) y -= p;
    return y;
}
PG_HD uint64_t advance_residue(uint64_t t0, uint64_t mi_lo, uint64_t r, uint64_t p) {
    if (mi_lo == 0) return t0;
    uint64_t s = mulmod_u64(mi_lo % p, r, p, 1.0 / (double)p);
    uint64_t y = t0 + s;
    return y >= p ? y - p : y;
}

// Calls emit(mi, y) for every mi in [mi_lo, mi_hi), ascending, with
// y = (y0 + (mi - mi_lo) * a) mod p <= two_sl, where y0 = y(mi_lo).
// Needs p > 2 * (two_sl + 1) and 0 < a < p.
template <typename T, typename Emit>
PG_HD void enumerate_hits(T p, T a, T y, uint64_t mi_lo, uint64_t mi_hi, T two_sl, Emit &emit) {
    uint64_t mi = mi_lo;
    if (mi >= mi_hi) return;
    if (y > two_sl) {
        uint64_t k;
        T v;
        modsearch_any(p, a, p - y, p - y + two_sl, k, v);
        mi += k;
        if (mi >= mi_hi) return;
        y = y - (p - v);  // (y + v) mod p with v in [p - y, p - y + two_sl]
    }
    const ThreeGap<T> g = three_gap<T>(p, a, two_sl + 1);
    if (g.up > two_sl || g.dn > two_sl) return;  // unreachable for prime p > 2(two_sl+1)
    for (;;) {
        emit(mi, y);
        if (y + g.up <= two_sl) {
            mi += g.kp;
            y += g.up;
        } else if (y >= g.dn) {
            mi += g.kn;
            y -= g.dn;
        } else {
            mi += (uint64_t)g.kp + g.kn;
            y = (y + g.up) - g.dn;
        }
        if (mi >= mi_hi) return;
    }
}

// Every hit with mi in [mi_lo, mi_hi), from y0 = y(mi_lo): first entry by
// the continued fraction, then the rotation steps of its last level.
template <typename T, typename Emit>
PG_HD void enumerate_hits_cf(T p, T a, T y0, uint64_t mi_lo, uint64_t mi_hi, T two_sl, Emit &emit) {
    const T w = two_sl + 1;
    const Entry<T> e = first_entry<T>(p, a, w, y0);
    if (e.y >= w) return;  // unreachable for prime p > 2w
    uint64_t mi = mi_lo + e.t;
    T y = e.y;
    const T C = e.g.up + e.g.dn;
    while (mi < mi_hi) {
        if (y < w) emit(mi, y);
        y += e.g.up;
        if (y >= C) {
            y -= C;
            mi += e.g.kn;
        } else {
            mi += e.g.kp;
        }
    }
}

// ---------------------------------------------------------------------------
// one prime's hits (modulo_search_euclid_all_large) spread over the grid.
// The continued fraction gives the first hit (mi0, y0) and the rotation
// after it: by `up` on a circle of C = up + dn points, a step costing kp
// (no wrap) or kn (wrap) in mi, every point below w = 2*SL+1 a hit.  Step n
// has the closed form Y = y0 + n*up, W = floor(Y / C) wraps, residue Y - W*C,
// mi = mi0 + (n - W)*kp + W*kn, so threads start their runs of steps
// anywhere.  Every CTA redoes the O(log p) set-up.
struct HitWalk {
    uint64_t mi0, y0, up, dn, kp, kn, w;
    uint64_t steps;  // upper bound on the steps with mi < max_mi
};

PG_HD bool hit_walk(uint64_t M, uint32_t max_mi, uint32_t sl, uint64_t p, uint64_t r, HitWalk &hw) {
    const uint64_t w = 2ull * sl + 1;
    uint64_t y;  // y(0) = (r*M + SL) mod p
    if (p < 0xFFFFFFFFull) {
        y = (((M % p) * r) % p + sl) % p;
    } else {
        y = mulmod_u64(M % p, r, p, 1.0 / (double)p) + sl;
        if (y >= p) y -= p;
    }
    const Entry<uint64_t> e = first_entry<uint64_t>(p, r, w, y, max_mi);
    if (e.t >= max_mi || e.y >= w) return false;
    hw = HitWalk{e.t, e.y, e.g.up, e.g.dn, e.g.kp, e.g.kn, w,
                 rotation_steps_bound<uint64_t>(e.t, max_mi, e.g, p)};
    return true;
}

// Position of rotation step n, mi clamped to mi_hi (a walk stops there).
PG_HD void hit_walk_at(const HitWalk &hw, uint64_t n, uint64_t mi_hi, uint64_t &mi, uint64_t &y) {
    const uint64_t C = hw.up + hw.dn;
    const unsigned __int128 Y = (unsigned __int128)n * hw.up + hw.y0;
    const uint64_t W = (uint64_t)(Y / C);  // W <= n: y0 < C and up < C
    y = (uint64_t)(Y - (unsigned __int128)W * C);
    const unsigned __int128 m =
        (unsigned __int128)hw.mi0 + (unsigned __int128)(n - W) * hw.kp + (unsigned __int128)W * hw.kn;
    mi = m < mi_hi ? (uint64_t)m : mi_hi;
}

// Walks up to `len` steps from (mi, y) while mi < mi_hi; calls emit(mi, y)
// at each hit and returns the number of hits.
template <typename Emit>
PG_HD uint32_t hit_walk_run(const HitWalk &hw, uint64_t mi, uint64_t y, uint64_t len, uint64_t mi_hi,
                                 Emit emit) {
    uint32_t n = 0;
    for (uint64_t k = 0; k < len && mi < mi_hi; k++) {
        if (y < hw.w) {
            emit(mi, y);
            n++;
        }
        const bool wrap = y >= hw.dn;
        y = wrap ? y - hw.dn : y + hw.up;
        mi += wrap ? hw.kn : hw.kp;
    }
    return n;
}

}  // namespace pg
