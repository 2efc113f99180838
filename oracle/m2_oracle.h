/*
 * ORACLE -- test infrastructure only.
 *
 * A plain-C CPU restatement of the reference's combined_sieve method2 path
 * (sethtroisi/prime-gap), used by the tests, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg as the checker.  Nothing in the product links,
 * loads or calls this code.
 *
 * Parity pin: the restatement reproduces the reference's own golden md5 values
 * from misc/tests.sh:66-71 and EXTENDED.md:186-187 (tests/test_oracle_golden.py).
 */
#ifndef PG_M2_ORACLE_H
#define PG_M2_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint32_t p;             /* primorial P (P#) */
    uint32_t d;             /* divisor, K = P#/d */
    uint64_t mstart;        /* first m */
    uint64_t minc;          /* m in [mstart, mstart + minc) */
    uint32_t sieve_length;  /* SL: offsets X in [-SL, SL] */
    uint64_t max_prime;     /* absolute (the CLI takes millions) */
    int32_t compression;    /* 0 plain text, 1 RLE, 2 bitcompressed */
    int32_t threads;        /* OpenMP threads, >= 1 */
} pgo_job;

/* Status codes (negative = error). */
#define PGO_OK 0
#define PGO_EINVAL -1
#define PGO_ENOMEM -2
#define PGO_EABORT -3 /* a case where the reference itself aborts on an assert */

/*
 * Run method2 on `job` and return the unknowns file contents (malloc'd,
 * caller frees with pgo_free).  Follows prime_gap_parallel()
 * (combined_sieve.cpp:2014-2447).
 */
int pgo_method2(const pgo_job *job, char **out, size_t *out_len);

/* Run and write the file to `path`. */
int pgo_method2_file(const pgo_job *job, const char *path);

void pgo_free(void *ptr);

/* ---- pieces exposed for known-answer tests ---- */

/* _modulo_search_euclid_small (modulo_search.cpp:71-98). */
uint32_t pgo_modulo_search_euclid_small(uint32_t p, uint32_t a, uint32_t l, uint32_t r);
/* _modulo_search_euclid (modulo_search.cpp:101-129). */
uint64_t pgo_modulo_search_euclid(uint64_t p, uint64_t a, uint64_t l, uint64_t r);
/* _modulo_search_euclid_stack (modulo_search.cpp:131-193). */
uint64_t pgo_modulo_search_euclid_stack(uint64_t p, uint64_t a, uint64_t l, uint64_t r);

/*
 * modulo_search_euclid_all_large (modulo_search.cpp:339-376): writes up to
 * `cap` (mi, temp_mod) pairs; returns the total number of hits.
 */
size_t pgo_modulo_search_all_large(uint64_t M, uint32_t max_mi, uint64_t SL, uint64_t prime,
                                   uint64_t base_r, uint32_t *mi_out, uint64_t *mod_out,
                                   size_t cap);

/* K = P#/d as little-endian 32-bit limbs; returns the limb count or <0. */
int pgo_build_k(uint32_t p, uint32_t d, uint32_t *limbs, int cap);
/* K mod q for q < 2^63. */
uint64_t pgo_k_mod(const uint32_t *limbs, int n, uint64_t q);

/* All primes in [lo, hi] in ascending order; returns the count written. */
size_t pgo_primes(uint64_t lo, uint64_t hi, uint64_t *out, size_t cap);
/* Number of primes in [lo, hi]. */
size_t pgo_count_primes(uint64_t lo, uint64_t hi);

/*
 * Thresholds of calculate_thresholds_method2 (gap_common.cpp:345-375), the
 * valid-m count, coprime-X count and LAST_PRIME = prevprime(max_prime).
 */
typedef struct {
    uint64_t small_threshold;
    uint64_t medium_threshold;
    uint64_t last_prime;
    uint64_t valid_ms;
    uint64_t coprime_x;
    uint64_t prime_limit; /* largest prime any phase sieves with */
} pgo_plan;
int pgo_plan_job(const pgo_job *job, pgo_plan *plan);

/*
 * Definition check, independent of the phase split: for each (m, X) pair,
 * returns in `smallest_factor[i]` the smallest prime q <= prime_limit that
 * divides m*K + X, or 0 if there is none.  This is the trial-division spot
 * check of surviving and removed offsets.
 */
int pgo_trial_division(const pgo_job *job, const uint64_t *m, const int64_t *x, size_t n,
                       uint64_t *smallest_factor);

/*
 * The unknowns of every valid m as binary lists: row i (file order) has m[i],
 * n_prev[i] distances of -X unknowns then n_next[i] of +X unknowns, each side
 * nearest first, at dist[start[i] ...].  Free with pgo_lists_free.
 */
typedef struct {
    uint64_t rows;
    uint64_t *m;
    uint32_t *n_prev, *n_next;
    uint64_t *start;
    uint32_t *dist;
    uint64_t total;
} pgo_lists;

/* parse_unknown_line (gap_common.cpp:1186-1360) over a whole unknowns file of
 * any compression; PGO_EINVAL on any line the reference would assert on. */
int pgo_parse_unknowns(const pgo_job *job, const char *text, size_t len, pgo_lists *out);
/* The same lists straight from the sieve, without text. */
int pgo_method2_lists(const pgo_job *job, pgo_lists *out);
void pgo_lists_free(pgo_lists *l);

#ifdef __cplusplus
}
#endif
#endif
