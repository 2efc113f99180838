/*
 * libpgsieve -- GB300 (sm_103a) method2 combined sieve, C ABI.
 *
 * The reference (sethtroisi/prime-gap) has no library interface for this
 * path: its boundary is the combined_sieve process, whose entry point is
 * prime_gap_parallel(Config&) (combined_sieve.cpp:2014) writing the unknowns
 * file through save_unknowns_method2 (combined_sieve.cpp:1261).  This header
 * is the C boundary a host program (the bundled combined_sieve CLI, or a
 * ctypes/cgo/JNI binding) calls instead.  Plain pointers and sizes only.
 *
 * Errors are returned as negative status codes; the library never exits,
 * aborts or traps.  One context per device; calls on one context are
 * serialised internally.
 */
#ifndef PGSIEVE_H
#define PGSIEVE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGS_OK 0
#define PGS_EINVAL (-1)   /* job rejected by the reference's validation (exit(1) there) */
#define PGS_ENOMEM (-2)   /* device or host allocation failed */
#define PGS_ECUDA (-3)    /* CUDA runtime error (message in pgs_last_error) */
#define PGS_EABORT (-4)   /* a job the reference itself aborts on with an assert */
#define PGS_ENODEV (-5)   /* no usable CUDA device */
#define PGS_ETIMEOUT (-6) /* a bounded device-side wait gave up */

typedef struct pgs_ctx pgs_ctx;

/*
 * One method2 job: the Config fields combined_sieve reads
 * (gap_common.h:39-89).  max_prime is absolute (the CLI's --max-prime is in
 * millions, gap_common.cpp:937-939).  compression: 0 plain text (default),
 * 1 --rle, 2 --bitcompressed (Config::compression, gap_common.h:57-62).
 */
typedef struct {
    uint32_t p;
    uint32_t d;
    uint64_t mstart;
    uint64_t minc;
    uint32_t sieve_length;
    uint64_t max_prime;
    int32_t compression;
    int32_t reserved;
} pgs_job;

/* Stage indexes of pgs_result.ms_stage (device time from CUDA events). */
enum {
    PGS_STAGE_SETUP = 0,  /* host tables -> device */
    PGS_STAGE_PRIMES = 1, /* segmented sieve */
    PGS_STAGE_KMOD = 2,   /* K mod p */
    PGS_STAGE_LARGE = 3,  /* large-prime marks */
    PGS_STAGE_ROWS = 4,   /* small primes + merge + compaction */
    PGS_STAGE_TEXT = 5,   /* scan + formatting */
    PGS_STAGE_D2H = 6,    /* text -> host */
    PGS_NSTAGES = 8
};

typedef struct {
    char *text;            /* unknowns file contents; owned by the library */
    uint64_t text_len;
    uint64_t rows;         /* valid m = rows of the file */
    uint64_t primes;       /* sieving primes: primes <= prime_limit */
    uint64_t prime_limit;  /* largest number whose prime factors are sieved */
    uint64_t unknowns;     /* total unknown offsets */
    double ms_total;       /* device time from setup to the last stage */
    double ms_stage[PGS_NSTAGES];
    uint64_t launches;     /* kernels launched for this job */
    void *internal;        /* owner of `text`; do not touch */
} pgs_result;

/* Create a context on CUDA device `device`. */
int pgs_create(int device, pgs_ctx **out);
void pgs_destroy(pgs_ctx *ctx);
/* Human-readable description of the last error on this context. */
const char *pgs_last_error(pgs_ctx *ctx);
/* Use an external CUDA stream (cudaStream_t as void*); NULL restores the
 * context's own stream.  A job also runs part of its work on a second
 * stream of the context (the small primes that its rows read and, with more
 * than one prime window, the next window's primes and K mod p), which waits
 * on this stream before its first launch and which this stream waits on
 * before the job's rows: the job's work stays ordered after what came
 * before it on this stream and before what comes after. */
int pgs_set_stream(pgs_ctx *ctx, void *stream);
/* The stream the context launches on (cudaStream_t as void*). */
void *pgs_get_stream(pgs_ctx *ctx);

/*
 * Run one job end to end and return the unknowns file bytes (replaces
 * prime_gap_parallel + save_unknowns_method2, combined_sieve.cpp:2014-2447,
 * 1261-1445).  Output is byte-identical to the reference's file for the same
 * parameters.  Free with pgs_result_free.
 */
int pgs_method2(pgs_ctx *ctx, const pgs_job *job, pgs_result *out);

/*
 * The same job by the per-m path (replaces combined_sieve --method1:
 * prime_gap_search and save_unknowns_method1, combined_sieve.cpp:383-751).
 * The reference files every large prime under the next m it divides and
 * sieves m by m; here the large-prime phase runs twice, counting and then
 * filing each surviving (m, X) under its m, and each m's marks come from its
 * own bucket.  The bytes equal pgs_method2's (the reference checks its two
 * methods against each other, misc/tests.sh:62-67); slower, a cross-check.
 */
int pgs_method1(pgs_ctx *ctx, const pgs_job *job, pgs_result *out);
void pgs_result_free(pgs_result *r);

/*
 * Split form for callers that keep the job resident: pgs_prepare uploads the
 * job's tables, pgs_run runs every sieve stage on the device (no host
 * transfer) and leaves the text on the device; pgs_fetch copies it out.
 */
typedef struct pgs_prepared pgs_prepared;
int pgs_prepare(pgs_ctx *ctx, const pgs_job *job, pgs_prepared **out);
int pgs_run(pgs_ctx *ctx, pgs_prepared *prep, int record_stages);
int pgs_fetch(pgs_ctx *ctx, pgs_prepared *prep, pgs_result *out);
void pgs_prepared_free(pgs_prepared *prep);

/* Device time of each stage of the last pgs_run on `prep` (waits for it);
 * out has PGS_NSTAGES entries, *total the whole run. */
int pgs_stage_ms(pgs_ctx *ctx, pgs_prepared *prep, double *out, double *total);

/*
 * Measured integer multiply-add issue rate of this device (32-bit IMAD per
 * second), from a microbenchmark kernel of independent mad.lo.u32 chains.
 * The integer-pipe roofline denominator of the sieve kernels.
 */
int pgs_int_peak(pgs_ctx *ctx, double *imad_per_s);

/*
 * Derived job parameters, as the reference computes them: valid m count,
 * offsets coprime to K, SMALL/MEDIUM thresholds of
 * calculate_thresholds_method2 (gap_common.cpp:345-375), and the unknowns
 * file name of Args::gen_unknown_fn (gap_common.cpp:732-749).
 */
typedef struct {
    uint64_t valid_ms;
    uint64_t coprime_x;
    uint64_t small_threshold;
    uint64_t medium_threshold;
    uint64_t prime_limit;
    uint32_t k_bits;
    char filename[256];
} pgs_plan;
int pgs_plan_job(const pgs_job *job, pgs_plan *out);

/* ---- many jobs: batched and served ------------------------------------ */

/*
 * Prime table resident on the context: every prime up to `limit` (sorted,
 * 2^30-wide windows) and the small primes the row phase needs, generated
 * once and shared by every batched or served job.  Grows on demand.
 */
int pgs_table_reserve(pgs_ctx *ctx, uint64_t limit);

/*
 * Batched method2: many jobs of uneven P, d, minc, SL and max_prime at once.
 * Jobs share the resident prime table and run concurrently on `lanes` CUDA
 * streams (each with its own scratch); the whole batch is captured as one
 * CUDA graph on its first pgs_batch_run and replayed afterwards.  Outputs are
 * byte-identical to pgs_method2 for each job.
 */
typedef struct pgs_batch pgs_batch;
int pgs_batch_prepare(pgs_ctx *ctx, const pgs_job *jobs, int n, int lanes, pgs_batch **out);
/* Run every job; *ms receives the device time of the batch (may be NULL). */
int pgs_batch_run(pgs_ctx *ctx, pgs_batch *b, int use_graph, double *ms);
int pgs_batch_fetch(pgs_ctx *ctx, pgs_batch *b, int i, pgs_result *out);
void pgs_batch_free(pgs_batch *b);
/* Convenience: prepare, run once and fetch all n results into outs. */
int pgs_method2_batch(pgs_ctx *ctx, const pgs_job *jobs, int n, pgs_result *outs);

/*
 * Served method2: a request loop.  Submitted jobs are admitted, in arrival
 * order, as soon as a lane is free and their device footprint (bitset, lists,
 * text and tables) fits under hbm_budget bytes; admitted jobs run
 * concurrently and their results are copied back as each one finishes (a
 * lane takes its next job as soon as its kernels are done; the copy-back
 * runs on two separate threads and streams; the next request is derived and
 * its tables uploaded while every lane is still busy).  K mod p is cached per
 * (P, d) and prime window, within a quarter of hbm_budget, for requests that
 * follow.
 * While a server runs it owns the context: make no other calls on it.
 */
typedef struct pgs_server pgs_server;
typedef struct {
    uint64_t submitted, completed, failed;
    double p50_ms, p99_ms, mean_ms, max_ms; /* submit-to-result latency */
    double busy_s;                          /* first admission to last result */
    uint64_t peak_bytes;                    /* largest admitted footprint sum */
    uint64_t max_inflight;
    double host_prep_s;  /* host time deriving, uploading and launching jobs */
    double host_fetch_s; /* host time copying results back */
    uint64_t kmod_fills; /* (P, d, prime window) K mod p passes computed */
    uint64_t kmod_hits;  /* ... and reused from the cache */
    double host_derive_s, host_upload_s, host_launch_s; /* parts of host_prep_s */
    double pinned_alloc_s; /* part of host_fetch_s spent allocating pinned memory */
    uint64_t pinned_allocs;
    double device_alloc_s; /* host time in cudaMalloc (device buffer pool misses) */
    uint64_t device_allocs;
} pgs_server_stats;
int pgs_server_start(pgs_ctx *ctx, uint64_t hbm_budget, int lanes, pgs_server **out);
int pgs_server_submit(pgs_server *srv, const pgs_job *job, uint64_t *ticket);
/* Wait for a ticket's result (timeout_ms < 0: no limit).  Returns
 * PGS_ETIMEOUT if it is not done in time, or the job's own status. */
int pgs_server_wait(pgs_server *srv, uint64_t ticket, int timeout_ms, pgs_result *out,
                    double *latency_ms);
int pgs_server_stats_get(pgs_server *srv, pgs_server_stats *out);
/* Finish every submitted job, stop the loop and free the server. */
int pgs_server_stop(pgs_server *srv);

/* ---- unknowns as lists: the next consumer, without a text parse -------- */

/*
 * Per-m unknown lists in file order, as gap_stats builds them with
 * parse_unknown_line (gap_common.cpp:1186-1360) from run_gap_file
 * (gap_stats.cpp:1181-1290): row i is m[i] with n_prev[i] distances of the
 * -X unknowns then n_next[i] of the +X unknowns, each side nearest first, at
 * dist[start[i] ...].  Library-owned; free with pgs_unknowns_free.
 */
typedef struct {
    uint64_t rows;
    uint64_t *m;
    uint64_t *start;
    uint32_t *n_prev, *n_next;
    uint32_t *dist;
    uint64_t total; /* entries of dist */
    void *internal;
} pgs_unknowns;
/* The lists of a job after pgs_run, read off the device (no text is parsed;
 * for a bitcompressed job its device-resident text is decoded in place). */
int pgs_fetch_unknowns(pgs_ctx *ctx, pgs_prepared *prep, pgs_unknowns *out);
/* Parse the bytes of an unknowns file of the job (plain, RLE or
 * bitcompressed, per job->compression) on the device.  PGS_EINVAL for a
 * file whose line count or any line does not match the job (where the
 * reference asserts). */
int pgs_parse_unknowns(pgs_ctx *ctx, const pgs_job *job, const char *text, uint64_t len,
                       pgs_unknowns *out);
void pgs_unknowns_free(pgs_unknowns *u);

/* ---- probable-prime tests of the unknowns (the step after the sieve) ---- */

/*
 * Base-2 strong probable-prime test of count numbers, each n_limbs
 * little-endian 32-bit limbs at limbs[i * n_limbs ...]; out[i] = 1 for a
 * probable prime.  Replaces test_runner_t::run_test / kernel_miller_rabin
 * (miller_rabin.h:247-383) with the one base gap_test_gpu uses (ROUNDS = 1,
 * gap_test_gpu.cu:81); its squaring loop bound is kept (miller_rabin.h:231-243:
 * up to s squarings for N - 1 = d 2^s).  rounds must be 1.  Numbers up to 4092
 * bits; even numbers and numbers below 8 are answered on the host.
 */
int pgs_prp_test(pgs_ctx *ctx, const uint32_t *limbs, uint32_t n_limbs, size_t count, int rounds,
                 uint8_t *out);

typedef struct {
    uint32_t p, d;          /* K = p#/d */
    uint32_t sieve_length;  /* past it a side searches on without unknowns */
    float min_merit;        /* gap_test's --min-merit (the reference's default is 18) */
    int one_side_skip;      /* 1: gap_test_gpu's skip of the next side when the previous
                               gap's merit is below min_merit/2 - 2 (gap_test_gpu.cu:570-596);
                               0: both sides always (gap_test_simple) */
} pgs_gap_params;

typedef struct {
    int32_t prev_p, next_p;     /* distances from m*K to the nearest probable primes below
                                   and above; next_p = 0 when the next side was skipped */
    uint32_t p_tests, n_tests;  /* unknowns tested on each side, the found one included
                                   (every unknown of a side that ran past the sieve length) */
    uint32_t flags;             /* 1: prev past the sieve length, 2: next past it,
                                   4: next side skipped */
} pgs_gap_result;

typedef struct {
    uint64_t rounds;     /* device rounds (candidate selection, tests, resolution) */
    uint64_t prp_tests;  /* probable-prime tests run, speculative ones included */
    uint32_t limbs;      /* 32-bit limbs per number on the device */
} pgs_gap_stats;

/*
 * The prime gap around m*K for every row of lists: each side's unknowns tested
 * nearest first until a probable prime, then past the sieve length the first
 * probable prime beyond it (replaces gap_test_gpu's load / GPU / overflow
 * threads, gap_test_gpu.cu:213-640, and test_interval_cpu with
 * mpz_prevprime / mpz_nextprime, gap_test_common.cpp:128-181).  out has
 * lists->rows entries; stats may be NULL.  PGS_EINVAL for p, d or lists that do
 * not fit (m*K up to 4092 bits).
 */
int pgs_prp_gaps(pgs_ctx *ctx, const pgs_gap_params *params, const pgs_unknowns *lists,
                 pgs_gap_result *out, pgs_gap_stats *stats);
/* The same search over the lists of a job after pgs_run, in place on the
 * device (no host copy of the lists): out has one entry per valid m of the
 * job, in file order.  The job's own p, d and sieve length are used;
 * params gives min_merit and one_side_skip. */
int pgs_prp_gaps_prepared(pgs_ctx *ctx, pgs_prepared *prep, const pgs_gap_params *params,
                          pgs_gap_result *out, pgs_gap_stats *stats);

/* ---- the reference's number-theory kernels, batched on the device ---- */

/*
 * Primes in [lo, hi], ascending (replaces primesieve::iterator walks,
 * combined_sieve.cpp:1475-1502).  Writes min(count, cap) primes.
 */
int pgs_primes(pgs_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *out, size_t cap, size_t *count);

/* K mod q for each q (replaces mpz_fdiv_ui, combined_sieve.cpp:1497, 1856);
 * K given as little-endian 32-bit limbs; odd q < 2^46. */
int pgs_k_mod_p(pgs_ctx *ctx, const uint32_t *k_limbs, int n_limbs, const uint64_t *q, size_t n,
                uint64_t *out);

/* Smallest k >= 1 with l <= k*a mod p <= r, for each i (replaces
 * _modulo_search_euclid, modulo_search.cpp:101-129); p < 2^46. */
int pgs_modulo_search(pgs_ctx *ctx, const uint64_t *p, const uint64_t *a, const uint64_t *l,
                      const uint64_t *r, uint64_t *k_out, size_t n);

/*
 * Every mi < max_mi with (base_r*(M+mi) + SL) mod prime <= 2*SL, ascending,
 * with that residue (replaces modulo_search_euclid_all_large,
 * modulo_search.cpp:339-376).  Needs prime > 4*SL + 2.  Writes up to cap
 * pairs and the total count.  The walk after the first hit is spread over
 * the grid (runs of steps started from their closed form), so a prime just
 * above 4*SL + 2 with max_mi near 2^32 takes milliseconds, not one thread's
 * 10^9 steps.
 */
int pgs_large_hits(pgs_ctx *ctx, uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t prime,
                   uint64_t base_r, uint32_t *mi_out, uint64_t *mod_out, size_t cap,
                   size_t *count);

/*
 * pgs_large_hits that allocates nothing.  No counterpart in the reference.
 *
 * Same arguments, results and errors as pgs_large_hits, but the device hit
 * lists and counter live in a fixed file-scope device buffer instead of
 * per-call cudaMalloc/cudaFree.  For callers that must not allocate: a
 * query made on a second context while a batch or server keeps kernels in
 * flight on the same device (cudaFree waits for the whole device to go idle,
 * so every pgs_large_hits call would stall behind, and hold up, those jobs),
 * and callers running at their device-memory budget.
 *
 * Limit: cap <= 65536 hits per call; a larger cap returns PGS_EINVAL.  The
 * count written may still exceed cap (only cap pairs are written).
 * The buffer's address is looked up once per device on the first call
 * (cudaGetSymbolAddress, which may load the module): make that first call
 * before any stream capture on the device.  The buffer is shared by every
 * context on a device: calls that overlap in time race on it, so serialise
 * them (calls on one context are serialised by the context).  The cached
 * address, like every context's streams and buffers, does not survive a
 * cudaDeviceReset: do not reset a device while the library is in use on it.
 */
int pgs_large_hits_static(pgs_ctx *ctx, uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t prime,
                          uint64_t base_r, uint32_t *mi_out, uint64_t *mod_out, size_t cap,
                          size_t *count);

/*
 * Tuning: the launch knobs of the sieve kernels, picked per job class by
 * measurement on the live device.  No counterpart in the reference, whose
 * nearest analogue is the hand cost model calculate_thresholds_method2
 * (gap_common.cpp:345-375) choosing its phase thresholds per job.  Every
 * value gives the same output; only the time changes.
 */
typedef struct {
    uint32_t direct_steps;   /* large-prime walks of at most this many steps run in their
                                continued-fraction thread (default 24) */
    uint32_t item_steps;     /* steps per item when a walk is spread over its CTA: 32, 64
                                or 128 (default 64) */
    uint32_t heavy_steps;    /* walks of more steps get a CTA of their own (default 4096) */
    uint32_t rows_per_cta;   /* most rows per CTA of the small-prime kernel, 1..32
                                (default 16; shared memory may allow fewer) */
    uint32_t text_chunks;    /* chunks of pgs_method2's rows/text/copy pipeline, 1..4
                                (default 4) */
    uint32_t kmod_lsb_limbs; /* K mod p least significant limb first from this many limbs
                                (default 32) */
    uint32_t large_form;     /* large-prime kernel of a one-job run, two bits.  Bit 0: 0 =
                                CTAs pool their primes' walks as 64-step items (default),
                                1 = warps run alone and hand longer walks to a list walked
                                one warp per walk (faster for short walks, i.e. small
                                jobs).  Bits 1 and 2: K mod p of the large primes below
                                and above 2^32 is computed inside that kernel (K of at
                                most 1024 limbs) instead of in a launch of its own */
} pgs_tuning;

void pgs_tuning_default(pgs_tuning *out);
/* The job's tuning class,
 * "P<p>.SL<floor(log2 SL)>.minc<floor(log2 minc)>.mp<floor(log2 max_prime)>";
 * returns the length (without the NUL), or PGS_EINVAL if cap is too small. */
int pgs_tuning_class(const pgs_job *job, char *buf, size_t cap);
/* Knobs for the job's class on this context (PGS_EINVAL for values outside
 * the ranges above).  One-job runs prepared afterwards (pgs_prepare,
 * pgs_method2) use them; batched and served jobs keep the defaults. */
int pgs_tuning_set(pgs_ctx *ctx, const pgs_job *job, const pgs_tuning *t);
/* The knobs jobs of this class get: returns 1 when the class is tuned, 0
 * when it gets the defaults. */
int pgs_tuning_get(pgs_ctx *ctx, const pgs_job *job, pgs_tuning *out);
/* Load the file's entries for this device (by name); returns how many, or
 * PGS_EINVAL when the file cannot be read. */
int pgs_tuning_load(pgs_ctx *ctx, const char *path);
/* Write this context's entries, keeping other devices' lines of the file. */
int pgs_tuning_save(pgs_ctx *ctx, const char *path);
/*
 * Tune the job's class: the job is prepared once and run `reps` times per
 * candidate (device time of pgs_run, median; pgs_method2's pipeline for
 * text_chunks), one knob at a time from the defaults, keeping a change that
 * is at least 2 % faster; the pick is then timed against the defaults three
 * times alternately and kept only if it is at least 1 % faster.  Stores and
 * returns the result, and the median times with the defaults and with it.
 */
int pgs_tune(pgs_ctx *ctx, const pgs_job *job, int reps, pgs_tuning *out, double *ms_default,
             double *ms_tuned);

/* Library version string. */
const char *pgs_version(void);

#ifdef __cplusplus
}
#endif
#endif
