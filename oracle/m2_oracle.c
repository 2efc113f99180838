/*
 * ORACLE -- test infrastructure only (see m2_oracle.h).
 *
 * CPU restatement of combined_sieve method2 from sethtroisi/prime-gap.  Each
 * function names the reference lines it follows.  Differences from the
 * reference that cannot change the output, by design of the algorithm
 * (marking is an idempotent OR, so only the SET of (m, X, p) marks matters):
 *   - no METHOD2_WHEEL x-reindexing (combined_sieve.cpp:1124-1200): every X
 *     coprime to K gets a column; primes dividing the wheel are sieved per m
 *     like the other primes of d;
 *   - the 2310 pre-filters of the medium/large phases are folded into the
 *     is_m_coprime / is_offset_coprime checks they shortcut;
 *   - K mod p uses a reciprocal-based remainder (Moller & Granlund, "Improved
 *     division by invariant integers", IEEE TC 2011, Alg. 4) instead of GMP's
 *     mpz_fdiv_ui; both return the exact remainder.
 *   - prime iteration is an own segmented sieve of Eratosthenes, not
 *     primesieve.
 */
#include "m2_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

void pgo_free(void *ptr) { free(ptr); }

/* ------------------------------------------------------------------------ */
/* small helpers                                                             */

static int is_prime_small(uint64_t n) {
    if (n < 2) return 0;
    if (n % 2 == 0) return n == 2;
    for (uint64_t t = 3; t * t <= n; t += 2)
        if (n % t == 0) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* modulo search, modulo_search.cpp                                          */

/* modulo_search.cpp:71-98: smallest k >= 1 with l <= k*a mod p <= r. */
uint32_t pgo_modulo_search_euclid_small(uint32_t p, uint32_t a, uint32_t l, uint32_t r) {
    uint32_t delta = r - l;
    if (a > (p >> 1)) {
        l = l + delta;
        a = p - a;
        l = p - l;
    }
    uint32_t l_div = (l - 1) / a;
    uint32_t l_mod = l - l_div * a;
    uint32_t r_mod = l_mod + delta;
    if (r_mod >= a) return l_div + 1;

    uint32_t new_a = a - (p % a);
    uint64_t k = pgo_modulo_search_euclid_small(a, new_a, l_mod, r_mod);
    uint64_t tl = k * p + l;
    uint64_t mult = (tl - 1) / a + 1;
    return (uint32_t)mult;
}

/* modulo_search.cpp:101-129 */
uint64_t pgo_modulo_search_euclid(uint64_t p, uint64_t a, uint64_t l, uint64_t r) {
    if (p < 0xFFFFFFFFull) return pgo_modulo_search_euclid_small(p, a, l, r);
    uint64_t delta = r - l;
    if (a > (p >> 1)) {
        l = l + delta;
        a = p - a;
        l = p - l;
    }
    uint64_t l_div = (l - 1) / a;
    uint64_t l_mod = l - l_div * a;
    uint64_t r_mod = l_mod + delta;
    if (r_mod >= a) return l_div + 1;
    uint64_t new_a = a - (p % a);
    uint64_t k = pgo_modulo_search_euclid(a, new_a, l_mod, r_mod);
    u128 tl = (u128)p * k + l;
    return (uint64_t)((tl - 1) / a + 1);
}

/* modulo_search.cpp:131-193: the explicit-stack form used by the sieve. */
uint64_t pgo_modulo_search_euclid_stack(uint64_t p, uint64_t a, uint64_t l, uint64_t r) {
    if (p < 0xFFFFFFFFull) return pgo_modulo_search_euclid_small(p, a, l, r);
    uint64_t stack[4 * 64];
    int sp = 0;
    uint64_t k = 0;
    uint64_t delta = r - l;
    for (;;) {
        if (a > (p >> 1)) {
            l = l + delta;
            a = p - a;
            l = p - l;
        }
        uint64_t l_div = (l - 1) / a;
        uint64_t l_mod = l - l_div * a;
        uint64_t r_mod = l_mod + delta;
        if (r_mod >= a) {
            k = l_div + 1;
            break;
        }
        uint64_t div = p / a;
        uint64_t rem = p - div * a;
        uint64_t new_a = a - rem;
        stack[sp++] = rem;
        stack[sp++] = div;
        stack[sp++] = a;
        stack[sp++] = l;
        p = a;
        a = new_a;
        l = l_mod;
    }
    while (sp > 0) {
        uint64_t sl = stack[--sp];
        uint64_t sa = stack[--sp];
        uint64_t sdiv = stack[--sp];
        uint64_t srem = stack[--sp];
        uint64_t k_1 = k * sdiv + 1;
        uint64_t k_2 = (uint64_t)(((u128)k * srem + sl - 1) / sa);
        k = k_1 + k_2;
    }
    return k;
}

/*
 * modulo_search.cpp:339-376 (modulo_search_euclid_all_large), with the
 * callback replaced by the caller's loop: returns the next hit at or after
 * `*mi` (temp_mod in *modulo) or 0 when the range is exhausted.
 */
typedef struct {
    uint64_t prime, base_r, initial_modulo, modulo, mi;
    uint32_t max_mi, two_sl;
} all_large_state;

static void all_large_init(all_large_state *s, uint64_t M, uint32_t max_mi, uint64_t SL,
                           uint64_t prime, uint64_t base_r) {
    s->prime = prime;
    s->base_r = base_r;
    s->mi = 0;
    s->modulo = (uint64_t)(((u128)base_r * M + SL) % prime);
    s->initial_modulo = s->modulo;
    s->two_sl = (uint32_t)(SL << 1);
    s->max_mi = max_mi;
}

static int all_large_next(all_large_state *s, uint32_t *mi_out, uint64_t *mod_out) {
    for (;;) {
        if (s->modulo <= s->two_sl) {
            if (s->mi >= s->max_mi) return 0;
            *mi_out = (uint32_t)s->mi;
            *mod_out = s->modulo;
            s->mi += 1;
            if (s->mi >= s->max_mi) {
                s->modulo = s->prime; /* force exit on the next call */
                s->mi = s->max_mi;
                return 1;
            }
            s->modulo += s->base_r;
            if (s->modulo >= s->prime) s->modulo -= s->prime;
            return 1;
        }
        if (s->mi >= s->max_mi) return 0;
        uint64_t low = s->prime - s->modulo;
        uint64_t high = low + s->two_sl;
        s->mi += pgo_modulo_search_euclid_stack(s->prime, s->base_r, low, high);
        if (s->mi >= s->max_mi) return 0;
        s->modulo = (uint64_t)(((u128)s->base_r * s->mi + s->initial_modulo) % s->prime);
    }
}

size_t pgo_modulo_search_all_large(uint64_t M, uint32_t max_mi, uint64_t SL, uint64_t prime,
                                   uint64_t base_r, uint32_t *mi_out, uint64_t *mod_out,
                                   size_t cap) {
    all_large_state s;
    all_large_init(&s, M, max_mi, SL, prime, base_r);
    size_t n = 0;
    uint32_t mi;
    uint64_t md;
    while (all_large_next(&s, &mi, &md)) {
        if (n < cap) {
            mi_out[n] = mi;
            mod_out[n] = md;
        }
        n++;
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* K = P#/d and K mod q                                                       */

/* init_K (gap_common.cpp:116-121): product of the primes <= P not dividing d. */
int pgo_build_k(uint32_t p, uint32_t d, uint32_t *limbs, int cap) {
    if (p < 2 || d == 0 || cap < 1) return PGO_EINVAL;
    int n = 1;
    limbs[0] = 1;
    uint32_t rest = d;
    for (uint32_t q = 2; q <= p; q++) {
        if (!is_prime_small(q)) continue;
        if (rest % q == 0) {
            rest /= q;
            continue;
        }
        uint64_t carry = 0;
        for (int i = 0; i < n; i++) {
            uint64_t t = (uint64_t)limbs[i] * q + carry;
            limbs[i] = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) {
            if (n >= cap) return PGO_ENOMEM;
            limbs[n++] = (uint32_t)carry;
        }
    }
    /* d must divide P# exactly (gap_common.cpp:119 asserts it). */
    if (rest != 1) return PGO_EINVAL;
    if (n == 1 && limbs[0] <= 1) return PGO_EINVAL; /* gap_common.cpp:120 */
    return n;
}

/* Reciprocal of a normalized 64-bit divisor: floor((2^128-1)/dn) - 2^64. */
static uint64_t mg_reciprocal(uint64_t dn) {
    u128 num = ~(u128)0;
    return (uint64_t)(num / dn - ((u128)1 << 64));
}

/* One step of Moller-Granlund Alg. 4: remainder of (u1*2^64 + u0) / dn, u1 < dn. */
static inline uint64_t mg_rem(uint64_t u1, uint64_t u0, uint64_t dn, uint64_t v) {
    u128 q = (u128)v * u1;
    q += ((u128)u1 << 64) | u0;
    uint64_t q1 = (uint64_t)(q >> 64) + 1;
    uint64_t q0 = (uint64_t)q;
    uint64_t r = u0 - q1 * dn;
    if (r > q0) r += dn;
    if (r >= dn) r -= dn;
    return r;
}

/* mpz_fdiv_ui(K, q) as used at combined_sieve.cpp:1497, 1856. */
static inline uint64_t k_word(const uint32_t *limbs, int n, int i) {
    if (i < 0 || 2 * i >= n) return 0;
    uint64_t lo = limbs[2 * i];
    uint64_t hi = (2 * i + 1 < n) ? limbs[2 * i + 1] : 0;
    return lo | (hi << 32);
}

uint64_t pgo_k_mod(const uint32_t *limbs, int n, uint64_t q) {
    /* remainder of (K << s) by the normalized divisor q << s, then >> s */
    int s = __builtin_clzll(q);
    uint64_t dn = q << s;
    uint64_t v = mg_reciprocal(dn);
    int words = (n + 1) / 2;
    uint64_t r = 0;
    for (int i = words; i >= 0; i--) {
        uint64_t hi = k_word(limbs, n, i), lo = k_word(limbs, n, i - 1);
        uint64_t sw = s ? (hi << s) | (lo >> (64 - s)) : hi;
        r = mg_rem(r, sw, dn, v);
    }
    return r >> s;
}

/* mpz_invert(K mod q) for prime q (combined_sieve.cpp:1674-1686). */
static uint64_t inv_mod(uint64_t a, uint64_t q) {
    int64_t t = 0, nt = 1;
    uint64_t r = q, nr = a % q;
    while (nr) {
        uint64_t quo = r / nr;
        int64_t tmp = t - (int64_t)quo * nt;
        t = nt;
        nt = tmp;
        uint64_t rtmp = r - quo * nr;
        r = nr;
        nr = rtmp;
    }
    if (t < 0) t += (int64_t)q;
    return (uint64_t)t;
}

/* ------------------------------------------------------------------------ */
/* prime generation: segmented sieve of Eratosthenes over odd numbers          */

typedef struct {
    uint32_t *p; /* odd base primes */
    size_t n;
} base_primes;

static int base_primes_init(base_primes *b, uint64_t limit) {
    /* odd primes <= limit */
    if (limit < 3) limit = 3;
    uint8_t *c = calloc(limit + 1, 1);
    if (!c) return PGO_ENOMEM;
    size_t cap = 1024, n = 0;
    uint32_t *p = malloc(cap * sizeof(uint32_t));
    for (uint64_t i = 3; i <= limit; i += 2) {
        if (c[i]) continue;
        if (n == cap) {
            cap *= 2;
            p = realloc(p, cap * sizeof(uint32_t));
        }
        p[n++] = (uint32_t)i;
        for (uint64_t j = i * i; j <= limit; j += 2 * i) c[j] = 1;
    }
    free(c);
    b->p = p;
    b->n = n;
    return PGO_OK;
}

static uint64_t isqrt_u64(uint64_t n) {
    uint64_t r = (uint64_t)sqrt((double)n);
    while (r * r > n) r--;
    while ((r + 1) * (r + 1) <= n) r++;
    return r;
}

/*
 * Primes in [lo, hi] (hi < 2^62) into out (cap entries) using scratch `dead`
 * of at least (hi-lo)/2+2 bytes; returns the number of primes.
 */
static size_t sieve_window(const base_primes *b, uint64_t lo, uint64_t hi, uint8_t *dead,
                           uint64_t *out, size_t cap) {
    size_t n = 0;
    if (hi < lo) return 0;
    if (lo <= 2 && 2 <= hi) {
        if (n < cap) out[n] = 2;
        n++;
    }
    uint64_t first = lo < 3 ? 3 : (lo | 1);
    if (first > hi) return n;
    uint64_t count = (hi - first) / 2 + 1;
    memset(dead, 0, count);
    for (size_t i = 0; i < b->n; i++) {
        uint64_t q = b->p[i];
        uint64_t sq = q * q;
        if (sq > hi) break;
        uint64_t start = sq;
        if (start < first) {
            start = (first + q - 1) / q * q;
            if ((start & 1) == 0) start += q;
        }
        for (uint64_t idx = (start - first) / 2; idx < count; idx += q) dead[idx] = 1;
    }
    for (uint64_t i = 0; i < count; i++) {
        if (!dead[i]) {
            if (n < cap) out[n] = first + 2 * i;
            n++;
        }
    }
    return n;
}

#define SEG_SPAN (1u << 21) /* numbers per segment */

size_t pgo_primes(uint64_t lo, uint64_t hi, uint64_t *out, size_t cap) {
    base_primes b;
    if (base_primes_init(&b, isqrt_u64(hi) + 1)) return 0;
    uint8_t *dead = malloc(SEG_SPAN / 2 + 2);
    size_t n = 0;
    for (uint64_t s = lo; s <= hi; s += SEG_SPAN) {
        uint64_t e = s + SEG_SPAN - 1;
        if (e > hi) e = hi;
        n += sieve_window(&b, s, e, dead, out ? out + (n < cap ? n : cap) : NULL,
                          n < cap ? cap - n : 0);
        if (e == hi) break;
    }
    free(dead);
    free(b.p);
    return n;
}

size_t pgo_count_primes(uint64_t lo, uint64_t hi) { return pgo_primes(lo, hi, NULL, 0); }

static uint64_t prev_prime_below(uint64_t n) { /* largest prime < n, mpz_prevprime */
    if (n <= 2) return 0;
    uint64_t c = n - 1;
    while (c >= 2) {
        int prime = 1;
        if (c % 2 == 0) prime = (c == 2);
        else
            for (uint64_t t = 3; t * t <= c; t += 2)
                if (c % t == 0) {
                    prime = 0;
                    break;
                }
        if (prime) return c;
        c--;
    }
    return 0;
}

static uint64_t next_prime_above(uint64_t n) { /* smallest prime > n */
    uint64_t c = n + 1;
    while (!is_prime_small(c)) c++;
    return c;
}

/* ------------------------------------------------------------------------ */
/* job setup: Cached (combined_sieve.cpp:1097-1230), is_coprime_and_valid_m   */
/* (gap_common.cpp:307-342), thresholds (gap_common.cpp:345-375)               */

typedef struct {
    pgo_job job;
    uint32_t K[640];
    int K_n;
    int K_odd;
    uint64_t last_prime;
    uint64_t small_threshold, medium_threshold, small_limit;
    uint32_t sl, interval;
    /* m tables */
    uint8_t *is_m_coprime; /* minc */
    int32_t *m_reindex;    /* minc */
    uint32_t *valid_mi;
    uint64_t valid_ms;
    /* X tables */
    uint8_t *is_offset_coprime; /* interval */
    uint32_t *x_reindex;        /* interval, 0 = not coprime */
    uint32_t *coprime_x;
    uint64_t coprime_count;
    /* composite bits: row = mii, column = x_reindex (1-based) */
    uint64_t words_per_row;
    uint64_t *composite;
} m2_state;

static void state_free(m2_state *s) {
    free(s->is_m_coprime);
    free(s->m_reindex);
    free(s->valid_mi);
    free(s->is_offset_coprime);
    free(s->x_reindex);
    free(s->coprime_x);
    free(s->composite);
}

static int validate_job(const pgo_job *j) {
    /* Args::argparse validation (gap_common.cpp:1007-1094) and main()'s
     * sieve_length window (combined_sieve.cpp:97-103). */
    if (j->p < 2 || !is_prime_small(j->p)) return PGO_EINVAL;
    if (j->d == 0 || j->mstart == 0 || j->minc == 0) return PGO_EINVAL;
    if (j->mstart + j->minc > 10000000001ull) return PGO_EINVAL;
    if (j->minc >= 0x7FFFFFFFull) return PGO_EINVAL;
    if (j->max_prime > 40000000000000ull || j->max_prime < 3) return PGO_EINVAL;
    if ((uint64_t)j->sieve_length < 6ull * j->p || (uint64_t)j->sieve_length > 22ull * j->p)
        return PGO_EINVAL;
    if (j->compression < 0 || j->compression > 2) return PGO_EINVAL;
    return PGO_OK;
}

static int state_init(m2_state *s, const pgo_job *job) {
    memset(s, 0, sizeof(*s));
    s->job = *job;
    int rc = validate_job(job);
    if (rc) return rc;
    s->K_n = pgo_build_k(job->p, job->d, s->K, 640);
    if (s->K_n < 0) return s->K_n;
    s->K_odd = s->K[0] & 1;
    s->sl = job->sieve_length;
    s->interval = 2 * s->sl + 1;
    /* combined_sieve.cpp:2030-2042 */
    s->last_prime = prev_prime_below(job->max_prime);

    const uint64_t minc = job->minc, ms = job->mstart;
    const uint32_t D = job->d;
    /* gap_common.cpp:307-342 */
    s->is_m_coprime = malloc(minc);
    s->m_reindex = malloc(minc * sizeof(int32_t));
    if (!s->is_m_coprime || !s->m_reindex) return PGO_ENOMEM;
    memset(s->is_m_coprime, 1, minc);
    for (uint32_t q = 2; q <= job->p; q++) {
        if (!is_prime_small(q) || D % q) continue;
        uint64_t first = (q - (ms % q)) % q;
        for (uint64_t mi = first; mi < minc; mi += q) s->is_m_coprime[mi] = 0;
    }
    uint64_t cnt = 0;
    for (uint64_t mi = 0; mi < minc; mi++) cnt += s->is_m_coprime[mi];
    s->valid_ms = cnt;
    if (cnt == 0) return PGO_EABORT; /* thresholds divide by valid_ms */
    s->valid_mi = malloc((cnt ? cnt : 1) * sizeof(uint32_t));
    cnt = 0;
    for (uint64_t mi = 0; mi < minc; mi++) {
        if (s->is_m_coprime[mi]) {
            s->m_reindex[mi] = (int32_t)cnt;
            s->valid_mi[cnt++] = (uint32_t)mi;
        } else {
            s->m_reindex[mi] = -1;
        }
    }

    /* combined_sieve.cpp:1143-1169: X coprime to K */
    s->is_offset_coprime = malloc(s->interval);
    s->x_reindex = calloc(s->interval, sizeof(uint32_t));
    memset(s->is_offset_coprime, 1, s->interval);
    for (uint32_t q = 2; q <= job->p; q++) {
        if (!is_prime_small(q) || D % q == 0) continue;
        uint32_t first = s->sl % q;
        for (uint32_t x = first; x < s->interval; x += q) s->is_offset_coprime[x] = 0;
    }
    uint64_t cc = 0;
    for (uint32_t x = 0; x < s->interval; x++) cc += s->is_offset_coprime[x];
    s->coprime_count = cc;
    s->coprime_x = malloc((cc ? cc : 1) * sizeof(uint32_t));
    cc = 0;
    for (uint32_t x = 0; x < s->interval; x++) {
        if (s->is_offset_coprime[x]) {
            s->coprime_x[cc++] = x;
            s->x_reindex[x] = (uint32_t)cc;
        }
    }

    /* gap_common.cpp:345-375, same float/double/integer conversions */
    {
        uint32_t sieve_interval = s->interval;
        double sm = log(8) * (double)job->minc / (double)s->valid_ms;
        float SMALL_MULT = (float)(8.0 > sm ? 8.0 : sm);
        uint64_t MEDIUM_CROSSOVER_SMALL =
            (uint64_t)(1.0 * (double)s->coprime_count * (double)job->minc / (double)s->valid_ms);
        float M_PER_P_CROSSOVER =
            (float)(1.0 * (double)job->minc * sieve_interval / (double)s->coprime_count);
        double mm = 0.65 * log2((double)(M_PER_P_CROSSOVER / (float)s->coprime_count));
        float MEDIUM_MULT = (float)(1.9 > mm ? 1.9 : mm);
        uint64_t MEDIUM_CROSSOVER_SEARCH = (uint64_t)(MEDIUM_MULT * M_PER_P_CROSSOVER);
        uint64_t SMALL = (uint64_t)SMALL_MULT * sieve_interval;
        if (MEDIUM_CROSSOVER_SMALL < SMALL) SMALL = MEDIUM_CROSSOVER_SMALL;
        if (SMALL < sieve_interval) SMALL = sieve_interval + 1;
        uint64_t MEDIUM = SMALL > MEDIUM_CROSSOVER_SEARCH ? SMALL : MEDIUM_CROSSOVER_SEARCH;
        if (MEDIUM > job->max_prime) MEDIUM = job->max_prime;
        s->small_threshold = SMALL;
        s->medium_threshold = MEDIUM;
    }
    /* combined_sieve.cpp:2080-2082 */
    if (s->medium_threshold < s->small_threshold) return PGO_EABORT;
    /* the small phase sieves through the first prime > SMALL_THRESHOLD
     * (loop at combined_sieve.cpp:1481-1504) */
    s->small_limit = next_prime_above(s->small_threshold);

    s->words_per_row = (s->coprime_count + 1 + 63) / 64;
    size_t bytes = (size_t)s->valid_ms * s->words_per_row * sizeof(uint64_t);
    s->composite = calloc(bytes ? bytes : 8, 1);
    if (!s->composite) return PGO_ENOMEM;
    return PGO_OK;
}

int pgo_plan_job(const pgo_job *job, pgo_plan *plan) {
    m2_state s;
    int rc = state_init(&s, job);
    if (rc == PGO_OK || rc == PGO_EABORT) {
        plan->small_threshold = s.small_threshold;
        plan->medium_threshold = s.medium_threshold;
        plan->last_prime = s.last_prime;
        plan->valid_ms = s.valid_ms;
        plan->coprime_x = s.coprime_count;
        plan->prime_limit = s.small_limit > s.last_prime ? s.small_limit : s.last_prime;
    }
    state_free(&s);
    return rc;
}

static inline void mark(m2_state *s, uint64_t mii, uint32_t col) {
    uint64_t *w = &s->composite[mii * s->words_per_row + (col >> 6)];
    __atomic_fetch_or(w, 1ull << (col & 63), __ATOMIC_RELAXED);
}

static inline int is_marked(const m2_state *s, uint64_t mii, uint32_t col) {
    return (s->composite[mii * s->words_per_row + (col >> 6)] >> (col & 63)) & 1;
}

/* ------------------------------------------------------------------------ */
/* phases                                                                     */

/* method2_small_primes (combined_sieve.cpp:1450-1603) */
static void phase_small(m2_state *s) {
    const pgo_job *j = &s->job;
    const uint64_t limit = s->small_limit;
    uint64_t *pr = malloc((limit + 2) * sizeof(uint64_t));
    size_t np = pgo_primes(2, limit, pr, limit + 2);
    uint32_t *sp = malloc((np ? np : 1) * sizeof(uint32_t));
    uint32_t *sr = malloc((np ? np : 1) * sizeof(uint32_t));
    size_t n = 0;
    for (size_t i = 0; i < np; i++) {
        uint64_t q = pr[i];
        /* combined_sieve.cpp:1494-1499 */
        if (j->d % q == 0 || q > j->p) {
            sp[n] = (uint32_t)q;
            sr[n] = (uint32_t)pgo_k_mod(s->K, s->K_n, q);
            n++;
        }
    }
    free(pr);
    const uint32_t SL = s->sl, INTERVAL = s->interval;
    const uint32_t D = j->d;

#pragma omp parallel for schedule(static) num_threads(j->threads)
    for (int64_t mii = 0; mii < (int64_t)s->valid_ms; mii++) {
        uint64_t m = j->mstart + s->valid_mi[mii];
        int centerOdd = ((D & 1) == 0) && (m & 1);
        int lowIsEven = centerOdd == (int)(SL & 1);
        for (size_t i = 0; i < n; i++) {
            uint64_t a_prime = sp[i];
            uint64_t base_r = sr[i];
            uint64_t modulo = (base_r * m) % a_prime;
            uint32_t flip = (uint32_t)(modulo + a_prime - ((SL + 1) % a_prime));
            if (flip >= a_prime) flip -= (uint32_t)a_prime;
            uint32_t first = (uint32_t)a_prime - flip - 1;
            if (first >= INTERVAL) continue;
            uint32_t shift = (uint32_t)a_prime;
            if (a_prime > 2) {
                int evenFromLow = (first & 1) == 0;
                int firstIsEven = lowIsEven == evenFromLow;
                if (firstIsEven) first += (uint32_t)a_prime;
                shift *= 2;
            }
            for (uint64_t x = first; x < INTERVAL; x += shift) {
                uint32_t xii = s->x_reindex[x];
                if (xii) mark(s, (uint64_t)mii, xii);
            }
        }
    }
    free(sp);
    free(sr);
}

/* method2_medium_primes (combined_sieve.cpp:1606-1760) for one prime */
static void medium_prime(m2_state *s, uint64_t prime) {
    const pgo_job *j = &s->job;
    const uint64_t M_start = j->mstart, M_inc = j->minc;
    const uint64_t SL = s->sl;
    const int K_odd = s->K_odd;
    const uint64_t base_r = pgo_k_mod(s->K, s->K_n, prime);
    const int64_t inv_K = (int64_t)inv_mod(base_r, prime);
    const int64_t neg_inv_K = (int64_t)prime - inv_K;
    const int64_t m_start_shift = (int64_t)((prime - (M_start % prime)) % prime);
    const int64_t SL_shift = (int64_t)((SL * (uint64_t)inv_K) % prime);
    const int64_t mi_0_shift = (m_start_shift + SL_shift) % (int64_t)prime;
    const int64_t X_M_parity_check = (int64_t)((M_start + SL) & 1);
    for (uint64_t xi = 0; xi < s->coprime_count; xi++) {
        int64_t X = s->coprime_x[xi];
        int64_t mi_0 = (X * neg_inv_K + mi_0_shift) % (int64_t)prime;
        if (K_odd && ((X ^ mi_0) & 1) == X_M_parity_check) mi_0 += (int64_t)prime;
        uint64_t shift = prime << K_odd;
        for (uint64_t mi = (uint64_t)mi_0; mi < M_inc; mi += shift) {
            if (!s->is_m_coprime[mi]) continue;
            mark(s, (uint64_t)s->m_reindex[mi], (uint32_t)(xi + 1));
        }
    }
}

/* method2_large_primes (combined_sieve.cpp:1763-2011) for one prime */
static void large_prime(m2_state *s, uint64_t prime) {
    const pgo_job *j = &s->job;
    const uint64_t base_r = pgo_k_mod(s->K, s->K_n, prime);
    all_large_state st;
    all_large_init(&st, j->mstart, (uint32_t)j->minc, s->sl, prime, base_r);
    uint32_t mi;
    uint64_t temp_mod;
    while (all_large_next(&st, &mi, &temp_mod)) {
        uint32_t x = 2 * s->sl - (uint32_t)temp_mod; /* combined_sieve.cpp:1878 */
        if (!s->is_m_coprime[mi]) continue;
        uint32_t xii = s->x_reindex[x];
        if (!xii) continue;
        mark(s, (uint64_t)s->m_reindex[mi], xii);
    }
}

/* Runs fn over every prime in [lo, hi] in parallel segments. */
static void for_primes(m2_state *s, uint64_t lo, uint64_t hi,
                       void (*fn)(m2_state *, uint64_t)) {
    if (hi < lo) return;
    base_primes b;
    base_primes_init(&b, isqrt_u64(hi) + 1);
    const uint64_t span = SEG_SPAN;
    const int64_t nseg = (int64_t)((hi - lo) / span + 1);
#pragma omp parallel num_threads(s->job.threads)
    {
        uint8_t *dead = malloc(span / 2 + 2);
        uint64_t *buf = malloc((span / 2 + 2) * sizeof(uint64_t));
#pragma omp for schedule(dynamic, 1)
        for (int64_t g = 0; g < nseg; g++) {
            uint64_t a = lo + (uint64_t)g * span;
            uint64_t e = a + span - 1;
            if (e > hi) e = hi;
            size_t n = sieve_window(&b, a, e, dead, buf, span / 2 + 2);
            for (size_t i = 0; i < n; i++) fn(s, buf[i]);
        }
        free(dead);
        free(buf);
    }
    free(b.p);
}

/* ------------------------------------------------------------------------ */
/* save_unknowns_method2 (combined_sieve.cpp:1261-1445)                        */

typedef struct {
    char *p;
    size_t n, cap;
} sbuf;

static void sb_put(sbuf *b, const char *src, size_t len) {
    if (b->n + len > b->cap) {
        size_t nc = b->cap ? b->cap * 2 : 256;
        while (nc < b->n + len) nc *= 2;
        b->p = realloc(b->p, nc);
        b->cap = nc;
    }
    memcpy(b->p + b->n, src, len);
    b->n += len;
}
static void sb_char(sbuf *b, char c) { sb_put(b, &c, 1); }
static void sb_u64(sbuf *b, uint64_t v) {
    char t[24];
    int n = 0;
    do {
        t[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    char o[24];
    for (int i = 0; i < n; i++) o[i] = t[n - 1 - i];
    sb_put(b, o, (size_t)n);
}

static void format_row(const m2_state *s, uint64_t mii, sbuf *line, const uint32_t *prev_x,
                       const uint32_t *next_x, size_t nside, const uint8_t *d_primes_flag,
                       uint64_t neg_k_mod_d, const uint32_t *d_primes, int n_dprimes,
                       uint8_t *scratch) {
    const pgo_job *j = &s->job;
    const uint64_t m = j->mstart + s->valid_mi[mii];
    const int32_t SL = (int32_t)s->sl;
    (void)d_primes_flag;
    if (j->compression == 2) {
        /* combined_sieve.cpp:1327-1385 */
        memcpy(scratch, s->is_offset_coprime, s->interval);
        for (int t = 0; t < n_dprimes; t++) {
            uint64_t dq = d_primes[t];
            uint64_t first = (m * neg_k_mod_d + (uint64_t)SL) % dq;
            for (uint64_t mult = first; mult < s->interval; mult += dq) scratch[mult] = 0;
        }
        sbuf raw = {0};
        size_t unknowns = 0, bytes_written = 0;
        int bit = 0;
        unsigned char b = 1u << 7;
        for (uint64_t xi = 0; xi < s->coprime_count; xi++) {
            uint32_t x = s->coprime_x[xi];
            if (scratch[x] == 1) {
                unsigned char is_composite = (unsigned char)is_marked(s, mii, s->x_reindex[x]);
                b |= (unsigned char)(is_composite << bit);
                unknowns += !is_composite;
                bit++;
                if (bit == 7) {
                    bytes_written++;
                    bit = 0;
                    sb_char(&raw, (char)b);
                    b = 1u << 7;
                }
            }
        }
        if (bit != 0) {
            bytes_written++;
            sb_char(&raw, (char)b);
        }
        sb_u64(line, m);
        sb_put(line, " : ", 3);
        sb_u64(line, unknowns);
        sb_char(line, ' ');
        sb_u64(line, bytes_written);
        sb_put(line, " || ", 4);
        if (raw.n) sb_put(line, raw.p, raw.n);
        sb_char(line, '\n');
        free(raw.p);
        return;
    }

    /* plain (combined_sieve.cpp:1418-1431) or RLE (1396-1417) */
    sbuf body = {0};
    uint64_t found_side[2] = {0, 0};
    for (int side = 0; side <= 1; side++) {
        int sign = side == 0 ? -1 : 1;
        const uint32_t *xs = side == 0 ? prev_x : next_x;
        sb_char(&body, '|');
        if (j->compression == 1) {
            sb_char(&body, ' ');
            int last = SL;
            for (size_t i = 0; i < nside; i++) {
                int x = (int)xs[i];
                if (!is_marked(s, mii, s->x_reindex[x])) {
                    found_side[side]++;
                    int delta = sign * (x - last);
                    last = x;
                    sb_char(&body, (char)(unsigned char)(48 + (delta >> 7)));
                    sb_char(&body, (char)(unsigned char)(48 + (delta & 127)));
                }
            }
        } else {
            for (size_t i = 0; i < nside; i++) {
                int x = (int)xs[i];
                if (!is_marked(s, mii, s->x_reindex[x])) {
                    sb_char(&body, ' ');
                    sb_char(&body, side == 0 ? '-' : '+');
                    sb_u64(&body, (uint64_t)(sign * (x - SL)));
                    found_side[side]++;
                }
            }
        }
        sb_char(&body, side == 0 ? ' ' : '\n');
    }
    sb_u64(line, m);
    sb_put(line, " : ", 3);
    sb_char(line, '-');
    sb_u64(line, found_side[0]);
    sb_char(line, ' ');
    sb_char(line, '+');
    sb_u64(line, found_side[1]);
    sb_char(line, ' ');
    sb_put(line, body.p, body.n);
    free(body.p);
}

static int save_unknowns(const m2_state *s, char **out, size_t *out_len) {
    const pgo_job *j = &s->job;
    const uint32_t SL = s->sl;
    /* coprime_prev / coprime_next, heading outward from SL (1289-1300) */
    size_t nside = 0;
    uint32_t *prev_x = malloc((s->coprime_count / 2 + 1) * sizeof(uint32_t));
    uint32_t *next_x = malloc((s->coprime_count / 2 + 1) * sizeof(uint32_t));
    for (uint64_t xi = 0; xi < s->coprime_count; xi++) {
        uint32_t x = s->coprime_x[xi];
        if (x > SL) {
            uint32_t dist = x - SL;
            prev_x[nside] = SL - dist;
            next_x[nside] = SL + dist;
            nside++;
        }
    }
    /* factors of d and -K mod d (1305-1314) */
    uint32_t d_primes[16];
    int n_dprimes = 0;
    for (uint32_t q = 2; q <= j->p && n_dprimes < 16; q++)
        if (is_prime_small(q) && j->d % q == 0) d_primes[n_dprimes++] = q;
    uint64_t k_mod_d = pgo_k_mod(s->K, s->K_n, j->d);
    uint64_t neg_k_mod_d = (j->d - k_mod_d) % j->d; /* mpz_cdiv_ui */

    const int64_t rows = (int64_t)s->valid_ms;
    sbuf *lines = calloc((size_t)(rows ? rows : 1), sizeof(sbuf));
    if (!lines) return PGO_ENOMEM;
#pragma omp parallel num_threads(j->threads)
    {
        uint8_t *scratch = malloc(s->interval);
#pragma omp for schedule(dynamic, 16)
        for (int64_t mii = 0; mii < rows; mii++)
            format_row(s, (uint64_t)mii, &lines[mii], prev_x, next_x, nside, NULL, neg_k_mod_d,
                       d_primes, n_dprimes, scratch);
        free(scratch);
    }
    size_t total = 0;
    for (int64_t i = 0; i < rows; i++) total += lines[i].n;
    char *buf = malloc(total ? total : 1);
    if (!buf) return PGO_ENOMEM;
    size_t pos = 0;
    for (int64_t i = 0; i < rows; i++) {
        memcpy(buf + pos, lines[i].p, lines[i].n);
        pos += lines[i].n;
        free(lines[i].p);
    }
    free(lines);
    free(prev_x);
    free(next_x);
    *out = buf;
    *out_len = total;
    return PGO_OK;
}

/* ------------------------------------------------------------------------ */

/* prime_gap_parallel (combined_sieve.cpp:2014-2447) */
int pgo_method2(const pgo_job *job, char **out, size_t *out_len) {
    m2_state s;
    int rc = state_init(&s, job);
    if (rc) {
        state_free(&s);
        return rc;
    }
    if (s.job.threads < 1) s.job.threads = 1;
    phase_small(&s);
    /* medium: primes in (SMALL_THRESHOLD, MEDIUM_THRESHOLD] (2244-2396) */
    for_primes(&s, s.small_threshold + 1, s.medium_threshold, medium_prime);
    /* large: primes in (MEDIUM_THRESHOLD, LAST_PRIME] (1763-2011) */
    for_primes(&s, s.medium_threshold + 1, s.last_prime, large_prime);
    rc = save_unknowns(&s, out, out_len);
    state_free(&s);
    return rc;
}

int pgo_method2_file(const pgo_job *job, const char *path) {
    char *buf = NULL;
    size_t n = 0;
    int rc = pgo_method2(job, &buf, &n);
    if (rc) return rc;
    FILE *f = fopen(path, "wb");
    if (!f) {
        free(buf);
        return PGO_EINVAL;
    }
    fwrite(buf, 1, n, f);
    fclose(f);
    free(buf);
    return PGO_OK;
}

/* ------------------------------------------------------------------------ */

int pgo_trial_division(const pgo_job *job, const uint64_t *m, const int64_t *x, size_t n,
                       uint64_t *smallest_factor) {
    pgo_plan plan;
    int rc = pgo_plan_job(job, &plan);
    if (rc && rc != PGO_EABORT) return rc;
    uint32_t K[640];
    int kn = pgo_build_k(job->p, job->d, K, 640);
    if (kn < 0) return kn;
    for (size_t i = 0; i < n; i++) smallest_factor[i] = 0;
    const uint64_t hi = plan.prime_limit;
    base_primes b;
    base_primes_init(&b, isqrt_u64(hi) + 1);
    const uint64_t span = SEG_SPAN;
    const int64_t nseg = (int64_t)(hi / span + 1);
    int threads = job->threads > 0 ? job->threads : 1;
#pragma omp parallel num_threads(threads)
    {
        uint8_t *dead = malloc(span / 2 + 2);
        uint64_t *buf = malloc((span / 2 + 2) * sizeof(uint64_t));
#pragma omp for schedule(dynamic, 1)
        for (int64_t g = 0; g < nseg; g++) {
            uint64_t a = (uint64_t)g * span;
            uint64_t e = a + span - 1;
            if (e > hi) e = hi;
            size_t np = sieve_window(&b, a, e, dead, buf, span / 2 + 2);
            for (size_t t = 0; t < np; t++) {
                uint64_t q = buf[t];
                uint64_t kr = pgo_k_mod(K, kn, q);
                for (size_t i = 0; i < n; i++) {
                    /* (m*K + X) mod q */
                    uint64_t v = (uint64_t)(((u128)(m[i] % q) * kr) % q);
                    int64_t xr = x[i] % (int64_t)q;
                    if (xr < 0) xr += (int64_t)q;
                    v = (v + (uint64_t)xr) % q;
                    if (v == 0) {
                        uint64_t cur = __atomic_load_n(&smallest_factor[i], __ATOMIC_RELAXED);
                        while ((cur == 0 || q < cur) &&
                               !__atomic_compare_exchange_n(&smallest_factor[i], &cur, q, 0,
                                                            __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                        }
                    }
                }
            }
        }
        free(dead);
        free(buf);
    }
    free(b.p);
    return PGO_OK;
}

/* ------------------------------------------------------------------------ */
/* unknowns as binary lists                                                   */

void pgo_lists_free(pgo_lists *l) {
    if (!l) return;
    free(l->m);
    free(l->n_prev);
    free(l->n_next);
    free(l->start);
    free(l->dist);
    memset(l, 0, sizeof(*l));
}

static int lists_alloc(pgo_lists *l, uint64_t rows, uint64_t cap) {
    memset(l, 0, sizeof(*l));
    l->rows = rows;
    l->m = malloc((rows + 1) * sizeof(uint64_t));
    l->n_prev = malloc((rows + 1) * sizeof(uint32_t));
    l->n_next = malloc((rows + 1) * sizeof(uint32_t));
    l->start = malloc((rows + 1) * sizeof(uint64_t));
    l->dist = malloc((cap + 1) * sizeof(uint32_t));
    if (!l->m || !l->n_prev || !l->n_next || !l->start || !l->dist) {
        pgo_lists_free(l);
        return PGO_ENOMEM;
    }
    return PGO_OK;
}

/* straight from the composite bits: a side's unknowns are the coprime
 * offsets heading outward from SL that are not marked (save_unknowns_method2,
 * combined_sieve.cpp:1387-1431, without the text) */
int pgo_method2_lists(const pgo_job *job, pgo_lists *out) {
    m2_state s;
    int rc = state_init(&s, job);
    if (rc) {
        state_free(&s);
        return rc;
    }
    if (s.job.threads < 1) s.job.threads = 1;
    phase_small(&s);
    for_primes(&s, s.small_threshold + 1, s.medium_threshold, medium_prime);
    for_primes(&s, s.medium_threshold + 1, s.last_prime, large_prime);
    const uint32_t SL = s.sl;
    uint32_t *dists = malloc((s.coprime_count / 2 + 1) * sizeof(uint32_t));
    size_t nside = 0;
    for (uint64_t xi = 0; xi < s.coprime_count; xi++)
        if (s.coprime_x[xi] > SL) dists[nside++] = s.coprime_x[xi] - SL;
    rc = lists_alloc(out, s.valid_ms, s.valid_ms * 2 * (uint64_t)nside);
    if (rc == PGO_OK) {
        uint64_t pos = 0;
        for (uint64_t mii = 0; mii < s.valid_ms; mii++) {
            out->m[mii] = s.job.mstart + s.valid_mi[mii];
            out->start[mii] = pos;
            for (int side = 0; side <= 1; side++) {
                uint32_t n = 0;
                for (size_t i = 0; i < nside; i++) {
                    const uint32_t x = side ? SL + dists[i] : SL - dists[i];
                    if (!is_marked(&s, mii, s.x_reindex[x])) {
                        out->dist[pos++] = dists[i];
                        n++;
                    }
                }
                if (side) out->n_next[mii] = n;
                else out->n_prev[mii] = n;
            }
        }
        out->total = pos;
    }
    free(dists);
    state_free(&s);
    return rc;
}

/* a cursor over one line */
typedef struct {
    const char *p, *end;
} cursor;

static void skip_ws(cursor *c) {
    while (c->p < c->end && (*c->p == ' ' || *c->p == '\t')) c->p++;
}
/* istream >> int64 */
static int read_i64(cursor *c, int64_t *v) {
    skip_ws(c);
    int neg = 0;
    if (c->p < c->end && (*c->p == '-' || *c->p == '+')) neg = *c->p++ == '-';
    if (c->p >= c->end || *c->p < '0' || *c->p > '9') return 0;
    int64_t x = 0;
    while (c->p < c->end && *c->p >= '0' && *c->p <= '9') x = x * 10 + (*c->p++ - '0');
    *v = neg ? -x : x;
    return 1;
}
/* istream >> std::string, compared with `tok` */
static int read_token(cursor *c, const char *tok) {
    skip_ws(c);
    const size_t n = strlen(tok);
    if ((size_t)(c->end - c->p) < n || memcmp(c->p, tok, n)) return 0;
    c->p += n;
    return c->p == c->end || *c->p == ' ' || *c->p == '\n';
}

/* parse_unknown_line (gap_common.cpp:1186-1360) for every line; the
 * BitArrayHelper tables (gap_common.cpp:1114-1180) come from the job */
int pgo_parse_unknowns(const pgo_job *job, const char *text, size_t len, pgo_lists *out) {
    m2_state s;
    int rc = state_init(&s, job);
    if (rc) {
        state_free(&s);
        return rc;
    }
    const uint32_t SL = s.sl, interval = s.interval;
    const int d_even = job->d % 2 == 0;
    /* coprime_X or coprime_X_even, and their flags */
    uint32_t *cx = malloc((s.coprime_count + 1) * sizeof(uint32_t));
    uint8_t *base_flags = calloc(interval, 1);
    size_t ncx = 0;
    for (uint64_t xi = 0; xi < s.coprime_count; xi++) {
        const uint32_t x = s.coprime_x[xi];
        if (d_even && ((x + SL) & 1)) continue; /* X = x - SL must be even */
        cx[ncx++] = x;
        base_flags[x] = 1;
    }
    uint32_t d_primes[16];
    int nd = 0;
    for (uint32_t q = 3; q <= job->p && nd < 16; q++)
        if (is_prime_small(q) && job->d % q == 0) d_primes[nd++] = q;
    const uint64_t neg_k_mod_d = (job->d - pgo_k_mod(s.K, s.K_n, job->d)) % job->d; /* mpz_cdiv_ui */
    uint8_t *flags = malloc(interval);
    /* a line has at most one unknown per listed offset */
    rc = lists_alloc(out, s.valid_ms, s.valid_ms * (uint64_t)(ncx + 1));
    const char *p = text, *end = text + len;
    uint64_t pos = 0;
    for (uint64_t mii = 0; rc == PGO_OK && mii < s.valid_ms; mii++) {
        const char *nl = memchr(p, '\n', (size_t)(end - p));
        if (!nl) {
            rc = PGO_EINVAL;
            break;
        }
        cursor c = {p, nl};
        p = nl + 1;
        int64_t m_test = -1;
        if (!read_i64(&c, &m_test) || m_test < 0 || !read_token(&c, ":")) {
            rc = PGO_EINVAL;
            break;
        }
        out->m[mii] = (uint64_t)m_test;
        out->start[mii] = pos;
        if (job->compression == 2) {
            memcpy(flags, base_flags, interval);
            const int center_odd = d_even && ((uint64_t)m_test & 1);
            const int low_is_even = center_odd == (int)(SL & 1);
            int64_t num = (int64_t)ncx;
            for (int t = 0; t < nd; t++) {
                const uint64_t q = d_primes[t];
                uint64_t first = ((uint64_t)m_test * neg_k_mod_d + SL) % q;
                const int even_from_low = (first & 1) == 0;
                if (low_is_even == even_from_low) first += q;
                for (uint64_t mult = first; mult < interval; mult += 2 * q)
                    if (flags[mult]) flags[mult] = 0, num--;
            }
            int64_t total = -1, bytes_check = -1;
            if (!read_i64(&c, &total) || total <= 0 || !read_i64(&c, &bytes_check) ||
                bytes_check != (num + 6) / 7 || !read_token(&c, "||") || c.p >= c.end || *c.p != ' ') {
                rc = PGO_EINVAL;
                break;
            }
            c.p++;
            if (c.end - c.p != bytes_check) {
                rc = PGO_EINVAL;
                break;
            }
            /* the low side comes farthest first in increasing x: collect, reverse */
            uint32_t np = 0, nn = 0;
            int bits = 0;
            size_t index = 0;
            unsigned char b = (unsigned char)c.p[0];
            for (size_t i = 0; i < ncx; i++) {
                const uint32_t x = cx[i];
                if (!flags[x]) continue;
                if (bits == 7) {
                    b = (unsigned char)c.p[++index];
                    bits = 0;
                }
                if ((b & 1) == 0) {
                    if (x <= SL) out->dist[pos + np++] = SL - x;
                    else nn++;
                }
                b >>= 1;
                bits++;
            }
            for (uint32_t i = 0; i < np / 2; i++) {
                uint32_t t = out->dist[pos + i];
                out->dist[pos + i] = out->dist[pos + np - 1 - i];
                out->dist[pos + np - 1 - i] = t;
            }
            bits = 0;
            index = 0;
            b = (unsigned char)c.p[0];
            uint32_t k = 0;
            for (size_t i = 0; i < ncx; i++) {
                const uint32_t x = cx[i];
                if (!flags[x]) continue;
                if (bits == 7) {
                    b = (unsigned char)c.p[++index];
                    bits = 0;
                }
                if ((b & 1) == 0 && x > SL) out->dist[pos + np + k++] = x - SL;
                b >>= 1;
                bits++;
            }
            if ((int64_t)(np + nn) != total) {
                rc = PGO_EINVAL;
                break;
            }
            out->n_prev[mii] = np;
            out->n_next[mii] = nn;
            pos += np + nn;
            continue;
        }
        int64_t ul = -1, uu = -1;
        if (!read_i64(&c, &ul) || !read_i64(&c, &uu) || !read_token(&c, "|") || c.p >= c.end ||
            *c.p != ' ') {
            rc = PGO_EINVAL;
            break;
        }
        ul = -ul;
        c.p++;
        if (ul < 0 || uu < 0) {
            rc = PGO_EINVAL;
            break;
        }
        for (int side = 0; side <= 1 && rc == PGO_OK; side++) {
            const int64_t n = side ? uu : ul;
            int64_t acc = 0;
            for (int64_t k = 0; k < n; k++) {
                if (job->compression == 1) {
                    if (c.end - c.p < 2) {
                        rc = PGO_EINVAL;
                        break;
                    }
                    const unsigned char a = (unsigned char)c.p[0], bb = (unsigned char)c.p[1];
                    c.p += 2;
                    acc += (int64_t)(a - 48) * 128 + (bb - 48);
                } else {
                    if (!read_i64(&c, &acc)) {
                        rc = PGO_EINVAL;
                        break;
                    }
                    if (side == 0) acc = -acc;
                }
                out->dist[pos++] = (uint32_t)acc;
            }
            if (rc == PGO_OK && side == 0) {
                if (!read_token(&c, "|") || c.p >= c.end || *c.p != ' ') {
                    rc = PGO_EINVAL;
                    break;
                }
                c.p++;
            }
        }
        out->n_prev[mii] = (uint32_t)ul;
        out->n_next[mii] = (uint32_t)uu;
    }
    if (rc == PGO_OK) out->total = pos;
    else pgo_lists_free(out);
    free(cx);
    free(base_flags);
    free(flags);
    state_free(&s);
    return rc;
}

/* ------------------------------------------------------------------------ */
#ifdef PGO_MAIN
/* m2_oracle -p P -d D --mstart M --minc N --sieve-length SL --max-prime MP(millions)
 *           [-t T] [--rle|--bitcompressed] -o OUT */
int main(int argc, char **argv) {
    pgo_job j = {0};
    j.threads = 1;
    const char *out = NULL;
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
        const char *v = i + 1 < argc ? argv[i + 1] : "0";
        if (!strcmp(a, "-p")) j.p = (uint32_t)atoi(v), i++;
        else if (!strcmp(a, "-d")) j.d = (uint32_t)atoi(v), i++;
        else if (!strcmp(a, "--mstart")) j.mstart = strtoull(v, 0, 10), i++;
        else if (!strcmp(a, "--minc")) j.minc = strtoull(v, 0, 10), i++;
        else if (!strcmp(a, "--sieve-length")) j.sieve_length = (uint32_t)atoi(v), i++;
        else if (!strcmp(a, "--max-prime")) j.max_prime = strtoull(v, 0, 10) * 1000000ull, i++;
        else if (!strcmp(a, "-t")) j.threads = atoi(v), i++;
        else if (!strcmp(a, "-o")) out = v, i++;
        else if (!strcmp(a, "--rle")) j.compression = 1;
        else if (!strcmp(a, "--bitcompressed")) j.compression = 2;
        else {
            fprintf(stderr, "unknown argument %s\n", a);
            return 1;
        }
    }
    if (!out) {
        fprintf(stderr, "need -o\n");
        return 1;
    }
    int rc = pgo_method2_file(&j, out);
    if (rc) fprintf(stderr, "m2_oracle failed: %d\n", rc);
    return rc ? 1 : 0;
}
#endif
