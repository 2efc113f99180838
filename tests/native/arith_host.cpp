// Host build of the device arithmetic (prime-gap_gb300/csrc/pg_arith.cuh) for
// CPU unit tests: the exact functions the kernels run, compiled by g++.
#include <cstddef>
#include <cstdint>

#include "pg_arith.cuh"

extern "C" {

uint64_t ah_modsearch(uint64_t p, uint64_t a, uint64_t l, uint64_t r, uint64_t *v) {
    pg::ModSearch64 s = pg::modsearch64(p, a, l, r);
    if (v) *v = s.v;
    return s.k;
}

void ah_three_gap(uint64_t p, uint64_t a, uint64_t w, uint64_t *out4) {
    if (p < 0xFFFFFFFFull) {
        pg::ThreeGap<uint32_t> g = pg::three_gap<uint32_t>((uint32_t)p, (uint32_t)a, (uint32_t)w);
        out4[0] = g.kp, out4[1] = g.up, out4[2] = g.kn, out4[3] = g.dn;
    } else {
        pg::ThreeGap<uint64_t> g = pg::three_gap<uint64_t>(p, a, w);
        out4[0] = g.kp, out4[1] = g.up, out4[2] = g.kn, out4[3] = g.dn;
    }
}

struct Collect {
    uint32_t *mi_out;
    uint64_t *mod_out;
    size_t cap, n;
    void operator()(uint64_t mi, uint64_t y) {
        if (n < cap) mi_out[n] = (uint32_t)mi, mod_out[n] = y;
        n++;
    }
    void operator()(uint64_t mi, uint64_t y, bool hit) {
        if (hit) (*this)(mi, y);
    }
};

// Hits of one prime over [0, max_mi), split into chunks of chunk_len values of
// mi the way the large-prime kernel splits them (chunk_len 0 = one chunk).
size_t ah_hits(uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t p, uint64_t r,
               uint32_t chunk_len, uint32_t *mi_out, uint64_t *mod_out, size_t cap) {
    Collect c{mi_out, mod_out, cap, 0};
    if (chunk_len == 0) chunk_len = max_mi;
    if (p < 0xFFFFFFFFull) {
        uint32_t pinv, r2;
        uint32_t p32 = (uint32_t)p, r32 = (uint32_t)r;
        (void)pinv, (void)r2;
        uint32_t t0 = (uint32_t)((((M % p32) * (uint64_t)r32) % p32 + SL) % p32);
        for (uint64_t lo = 0; lo < max_mi; lo += chunk_len) {
            uint64_t hi = lo + chunk_len < max_mi ? lo + chunk_len : max_mi;
            uint32_t y = pg::advance_residue(t0, lo, r32, p32);
            pg::enumerate_hits<uint32_t>(p32, r32, y, lo, hi, 2 * SL, c);
        }
    } else {
        uint64_t t0 = pg::mulmod_u64(M % p, r, p, 1.0 / (double)p) + SL;
        if (t0 >= p) t0 -= p;
        for (uint64_t lo = 0; lo < max_mi; lo += chunk_len) {
            uint64_t hi = lo + chunk_len < max_mi ? lo + chunk_len : max_mi;
            uint64_t y = pg::advance_residue(t0, lo, r, p);
            pg::enumerate_hits<uint64_t>(p, r, y, lo, hi, 2ull * SL, c);
        }
    }
    return c.n;
}

// Same, through the continued-fraction first entry and rotation steps.
size_t ah_hits_cf(uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t p, uint64_t r,
                  uint32_t chunk_len, uint32_t *mi_out, uint64_t *mod_out, size_t cap) {
    Collect c{mi_out, mod_out, cap, 0};
    if (chunk_len == 0) chunk_len = max_mi;
    if (p < 0xFFFFFFFFull) {
        uint32_t p32 = (uint32_t)p, r32 = (uint32_t)r;
        uint32_t t0 = (uint32_t)((((M % p32) * (uint64_t)r32) % p32 + SL) % p32);
        for (uint64_t lo = 0; lo < max_mi; lo += chunk_len) {
            uint64_t hi = lo + chunk_len < max_mi ? lo + chunk_len : max_mi;
            uint32_t y = pg::advance_residue(t0, lo, r32, p32);
            pg::enumerate_hits_cf<uint32_t>(p32, r32, y, lo, hi, 2 * SL, c);
        }
    } else {
        uint64_t t0 = pg::mulmod_u64(M % p, r, p, 1.0 / (double)p) + SL;
        if (t0 >= p) t0 -= p;
        for (uint64_t lo = 0; lo < max_mi; lo += chunk_len) {
            uint64_t hi = lo + chunk_len < max_mi ? lo + chunk_len : max_mi;
            uint64_t y = pg::advance_residue(t0, lo, r, p);
            pg::enumerate_hits_cf<uint64_t>(p, r, y, lo, hi, 2ull * SL, c);
        }
    }
    return c.n;
}

// Hits of one prime split the way the large-prime kernel splits them: first
// entry, then either a direct walk (bound <= direct) or items of item_steps
// steps started from the closed form.  Returns the hit count (hits in order).
size_t ah_hits_items(uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t p, uint64_t r,
                     uint32_t direct, uint32_t item_steps, uint32_t *mi_out, uint64_t *mod_out,
                     size_t cap) {
    Collect c{mi_out, mod_out, cap, 0};
    auto run = [&](auto p_, auto r_, auto t0) {
        using T = decltype(p_);
        const T w = (T)(2 * SL + 1);
        pg::Entry<T> e = pg::first_entry<T>(p_, r_, w, t0);
        if (e.t >= max_mi || e.y >= w) return;
        uint64_t bound = pg::rotation_steps_bound<T>(e.t, max_mi, e.g, p_);
        // the kernel's 32-bit walk forms, step costs clamped to max_mi
        const pg::ThreeGap<uint32_t> g = pg::gap32(e.g, max_mi);
        if (bound <= direct) {
            pg::return_walk32((uint32_t)e.t, (uint32_t)e.y, g, (uint32_t)w, max_mi, (uint32_t)bound, c);
            return;
        }
        uint64_t items = (bound + item_steps - 1) / item_steps;
        for (uint64_t it = 0; it < items; it++) {
            uint32_t y, mi;
            pg::rotation_at32((uint32_t)e.t, (uint32_t)e.y, g, (uint32_t)(it * item_steps), max_mi, y, mi);
            pg::return_walk32(mi, y, g, (uint32_t)w, max_mi, item_steps, c);
        }
    };
    if (p < 0xFFFFFFFFull) {
        uint32_t p32 = (uint32_t)p, r32 = (uint32_t)r;
        uint32_t t0 = (uint32_t)((((M % p32) * (uint64_t)r32) % p32 + SL) % p32);
        run(p32, r32, t0);
    } else {
        uint64_t t0 = pg::mulmod_u64(M % p, r, p, 1.0 / (double)p) + SL;
        if (t0 >= p) t0 -= p;
        run(p, r, t0);
    }
    return c.n;
}

// Parity-reduced walk of one prime (the large-prime kernel's walk): hits as
// (mi, x = X + SL) for d even (odd_d = 0) or d odd (odd_d = 1).
size_t ah_hits_parity(uint64_t M, uint32_t minc, uint32_t SL, uint64_t p, uint64_t r, int odd_d,
                      uint32_t *mi_out, uint64_t *x_out, size_t cap) {
    pg::WalkParams w{};
    if (!odd_d) {
        w.stride = 2;
        w.mi_base = (M & 1) ? 0 : 1;
        w.jmax = minc > w.mi_base ? (minc - w.mi_base + 1) / 2 : 0;
        w.c_add = SL / 2;
        w.w = 2 * (SL / 2) + 1;
        w.xc = 2 * (SL / 2) + SL;
    } else {
        uint32_t hi = (SL - 1) / 2, lo = (SL + 1) / 2;
        w.stride = 1;
        w.jmax = minc;
        w.c_add = hi;
        w.w = hi + lo + 1;
        w.xc = 2 * hi + 1 + SL;
        w.odd_d = 1;
    }
    w.m0 = M + w.mi_base;
    struct C {
        const pg::WalkParams &w;
        uint32_t *mi_out;
        uint64_t *x_out;
        size_t cap, n;
        void operator()(uint64_t j, uint64_t y) {
            if (n < cap) mi_out[n] = (uint32_t)(w.mi_base + w.stride * j), x_out[n] = w.xc - 2 * y;
            n++;
        }
        void operator()(uint64_t j, uint64_t y, bool hit) {
            if (hit) (*this)(j, y);
        }
    } c{w, mi_out, x_out, cap, 0};
    unsigned __int128 rh = pg::half_mod(r, p);
    uint64_t cc = w.c_add + (w.odd_d ? (p >> 1) + 1 : 0);
    uint64_t t0 = (uint64_t)((rh * (w.m0 % p) + cc) % p);
    uint64_t a = w.odd_d ? (uint64_t)rh : r;
    if (p < 0xFFFFFFFFull)
        pg::enumerate_hits_cf<uint32_t>((uint32_t)p, (uint32_t)a, (uint32_t)t0, 0, w.jmax,
                                        (uint32_t)(w.w - 1), c);
    else
        pg::enumerate_hits_cf<uint64_t>(p, a, t0, 0, w.jmax, (uint64_t)(w.w - 1), c);
    return c.n;
}

// first_entry: out = {t, y, kp, up, kn, dn}
void ah_first_entry(uint64_t p, uint64_t a, uint64_t w, uint64_t y0, uint64_t *out6) {
    if (p < 0xFFFFFFFFull) {
        auto e = pg::first_entry<uint32_t>((uint32_t)p, (uint32_t)a, (uint32_t)w, (uint32_t)y0);
        out6[0] = e.t, out6[1] = e.y, out6[2] = e.g.kp, out6[3] = e.g.up, out6[4] = e.g.kn,
        out6[5] = e.g.dn;
    } else {
        auto e = pg::first_entry<uint64_t>(p, a, w, y0);
        out6[0] = e.t, out6[1] = e.y, out6[2] = e.g.kp, out6[3] = e.g.up, out6[4] = e.g.kn,
        out6[5] = e.g.dn;
    }
}

// first_entry with an early stop at t_lim: out = {t, y, kp, up, kn, dn}
void ah_first_entry_lim(uint64_t p, uint64_t a, uint64_t w, uint64_t y0, uint64_t t_lim,
                        uint64_t *out6) {
    if (p < 0xFFFFFFFFull) {
        auto e = pg::first_entry<uint32_t>((uint32_t)p, (uint32_t)a, (uint32_t)w, (uint32_t)y0, t_lim);
        out6[0] = e.t, out6[1] = e.y, out6[2] = e.g.kp, out6[3] = e.g.up, out6[4] = e.g.kn,
        out6[5] = e.g.dn;
    } else {
        auto e = pg::first_entry<uint64_t>(p, a, w, y0, t_lim);
        out6[0] = e.t, out6[1] = e.y, out6[2] = e.g.kp, out6[3] = e.g.up, out6[4] = e.g.kn,
        out6[5] = e.g.dn;
    }
}

// least-significant-first K mod q: 4 interleaved 32-bit chains, or the 64-bit word chain
void ah_kmod4_lsb(const uint32_t *limbs, int n, const uint32_t *q4, uint32_t *out4, uint32_t *r2_4) {
    uint32_t pinv[4];
    pg::kmod32_lsb_multi<4>(limbs, n, q4, out4, pinv, r2_4);
}

uint64_t ah_kmod64_lsb(const uint32_t *limbs, int n, uint64_t q) { return pg::kmod64_lsb(limbs, n, q); }

// walk step and start residue from r = K mod p: out = {step, t0}
void ah_walk_start(uint64_t p, uint64_t r, uint64_t m0, uint32_t c_add, uint32_t odd_d, uint64_t *out2) {
    pg::WalkParams wk{};
    wk.m0 = m0;
    wk.c_add = c_add;
    wk.odd_d = odd_d;
    if (p < 0xFFFFFFFFull) {
        const uint32_t r1 = (uint32_t)((1ull << 32) % p);
        const uint32_t r2 = (uint32_t)(((uint64_t)r1 * r1) % p);
        uint32_t step, t0;
        pg::walk_start(wk, (uint32_t)p, (uint32_t)r, r2, step, t0);
        out2[0] = step, out2[1] = t0;
    } else {
        const uint64_t r1 = (0ull - p) % p;
        const uint64_t r2 = (uint64_t)(((unsigned __int128)r1 * r1) % p);
        uint64_t step, t0;
        pg::walk_start(wk, p, r, pg::neg_inv64(p), r2, step, t0);
        out2[0] = step, out2[1] = t0;
    }
}

uint64_t ah_kmod(const uint32_t *limbs, int n, uint64_t q) {
    if (q < 0x80000000ull) {
        uint32_t pinv, r2;
        return pg::kmod32(limbs, n, (uint32_t)q, pinv, r2);
    }
    return pg::kmod64(limbs, n, q);
}

// Four primes through the interleaved chains of the K mod p kernel.
void ah_kmod4(const uint32_t *limbs, int n, const uint32_t *q4, uint32_t *out4) {
    uint32_t pinv[4], r2[4];
    pg::kmod32_multi<4>(limbs, n, q4, out4, pinv, r2);
}

// (r * M + sl) mod p through the Montgomery path of the K mod p kernel.
uint32_t ah_start32(uint32_t r, uint64_t M, uint32_t sl, uint32_t p) {
    uint32_t pinv = pg::neg_inv32(p);
    uint32_t r1 = (0u - p) % p;
    uint32_t r2 = (uint32_t)(((uint64_t)r1 * r1) % p);
    return pg::start32(r, M, sl, p, pinv, r2);
}

uint64_t ah_mulmod(uint64_t a, uint64_t b, uint64_t p) { return pg::mulmod_u64(a, b, p, 1.0 / (double)p); }

// Montgomery reduction (R = 2^32) and -p^-1 mod 2^32 of the K mod p kernel.
uint32_t ah_redc32(uint64_t t, uint32_t p) { return pg::redc32(t, p, pg::neg_inv32(p)); }
uint32_t ah_neg_inv32(uint32_t p) { return pg::neg_inv32(p); }

// The grid form of pgs_large_hits (pg_tools.cu) run serially: the total
// from `threads` runs of consecutive steps, and the first `cap` hits written
// in order from the first 2*cap + 2 steps split over `cta` runs.  Returns
// the total count.
size_t ah_hits_grid(uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t p, uint64_t r, uint64_t threads,
                    uint64_t cta, uint32_t *mi_out, uint64_t *mod_out, size_t cap) {
    pg::HitWalk hw;
    if (!pg::hit_walk(M, max_mi, SL, p, r, hw)) return 0;
    size_t total = 0;
    const uint64_t run = (hw.steps + threads - 1) / threads;
    for (uint64_t t = 0; t < threads; t++) {
        const uint64_t n0 = t * run;
        if (n0 >= hw.steps) break;
        uint64_t mi, y;
        pg::hit_walk_at(hw, n0, max_mi, mi, y);
        total += pg::hit_walk_run(hw, mi, y, run < hw.steps - n0 ? run : hw.steps - n0, max_mi,
                                  [](uint64_t, uint64_t) {});
    }
    const uint64_t span = hw.steps < 2 * (uint64_t)cap + 2 ? hw.steps : 2 * (uint64_t)cap + 2;
    const uint64_t wrun = (span + cta - 1) / cta;
    uint64_t pos = 0;
    for (uint64_t t = 0; t < cta && cap; t++) {
        const uint64_t n0 = t * wrun;
        if (n0 >= span) break;
        uint64_t mi, y;
        pg::hit_walk_at(hw, n0, max_mi, mi, y);
        pg::hit_walk_run(hw, mi, y, wrun < span - n0 ? wrun : span - n0, max_mi, [&](uint64_t m, uint64_t v) {
            if (pos < cap) mi_out[pos] = (uint32_t)m, mod_out[pos] = v;
            pos++;
        });
    }
    return total;
}

// Two quotients by one divisor through the shared reciprocal (the
// continued fraction's division), with the reciprocal moved by `skew` ulps.
void ah_udiv2(uint32_t n1, uint32_t n2, uint32_t d, int skew, uint32_t *out2) {
    pg::udiv2_32(n1, n2, d, out2[0], out2[1], skew);
}

// The walk from (mi, y) over `steps` circle steps below mi_hi, both ways:
// circle steps (rotation_walk32) and hit to hit (return_walk32).  Writes the
// hits of each as (mi, y) pairs; returns 1 when the two lists agree.
struct HitList {
    uint32_t *out;
    size_t cap, n;
    void operator()(uint64_t mi, uint32_t y, bool hit) {
        if (!hit) return;
        if (n + 2 <= cap) out[n] = (uint32_t)mi, out[n + 1] = y;
        n += 2;
    }
};
int ah_return_walk_agrees(uint32_t mi, uint32_t y, uint32_t kp, uint32_t up, uint32_t kn, uint32_t dn,
                          uint32_t w, uint32_t mi_hi, uint32_t steps, uint32_t *buf, size_t cap, size_t *nhits) {
    const pg::ThreeGap<uint32_t> g{kp, up, kn, dn};
    HitList a{buf, cap / 2, 0}, b{buf + cap / 2, cap / 2, 0};
    pg::rotation_walk32(mi, y, g, w, mi_hi, steps, a);
    pg::return_walk32(mi, y, g, w, mi_hi, steps, b);
    *nhits = a.n / 2;
    if (a.n != b.n) return 0;
    for (size_t i = 0; i < a.n && i < cap / 2; i++)
        if (a.out[i] != b.out[i]) return 0;
    return 1;
}

void ah_pow64_128(uint64_t p, int skew, uint64_t *out2) { pg::pow64_128_mod(p, out2[0], out2[1], skew); }

uint64_t ah_neg_inv64(uint64_t p) { return pg::neg_inv64(p); }

void ah_udiv2f(uint32_t n1, uint32_t n2, uint32_t d, int skew, uint32_t *out2) {
    pg::udiv2f_32(n1, n2, d, out2[0], out2[1], skew);
}

void ah_udiv2_64(uint64_t n1, uint64_t n2, uint64_t d, int skew, uint64_t *out2) {
    pg::udiv2_64(n1, n2, d, out2[0], out2[1], skew);
}

// 2^32 mod p through the approximate reciprocal (K mod p setup).
uint32_t ah_pow32_mod(uint32_t p, int skew) { return pg::pow32_mod(p, skew); }

}
