// Internal declarations shared by the CUDA translation units of libpgsieve.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "pg_arith.cuh"

namespace pg {

// ---- prime sieve (pg_primes.cu) -------------------------------------------

// Odd numbers per sieve segment (one CTA): a 32 KiB shared bitmap.
constexpr uint32_t kSegBits = 32768u * 8u;
// Number line covered by one segment.
constexpr uint64_t kSegSpan = 2ull * kSegBits;

// Base primes for sieving windows up to `limit`: all odd primes <= sqrt(limit).
struct BasePrimes {
    uint32_t *d_primes = nullptr;  // device, ascending
    uint32_t count = 0;
    uint64_t covers = 0;  // windows up to covers are sievable
};

// Host-side: build base primes on the device for windows up to `limit`.
cudaError_t base_primes_build(BasePrimes &bp, uint64_t limit, cudaStream_t stream);
void base_primes_free(BasePrimes &bp);

// Upper bound on the number of primes in [lo, hi] (Brun-Titchmarsh,
// Montgomery-Vaughan form), plus slack; used to size output buffers.
uint64_t prime_count_bound(uint64_t lo, uint64_t hi);

// Sieve the odd primes in [lo, hi] (lo >= 3, hi - lo < 2^32) and append their
// offsets from `lo` (unordered) to d_out, counting into *d_count (device).
// cap = capacity of d_out.
cudaError_t sieve_window(const BasePrimes &bp, uint64_t lo, uint64_t hi, uint32_t *d_out,
                         uint64_t cap, unsigned long long *d_count, cudaStream_t stream);

// Sorted odd primes of [lo, hi] (hi - lo < 2^32) as offsets from lo; count
// to *d_count.  d_tmp: sieve_sorted_tmp_bytes(lo, hi) bytes of scratch.
uint64_t sieve_sorted_tmp_bytes(uint64_t lo, uint64_t hi);
cudaError_t sieve_window_sorted(const BasePrimes &bp, uint64_t lo, uint64_t hi, uint32_t *d_out,
                                uint64_t cap, unsigned long long *d_count, void *d_tmp,
                                cudaStream_t stream);
// d_out = {begin, end}: the indexes of the sorted list base + off[0..count)
// whose values lie in [lo_val, hi_val].
cudaError_t find_range(const uint32_t *d_off, uint64_t count, uint64_t base, uint64_t lo_val,
                       uint64_t hi_val, unsigned long long *d_out, cudaStream_t stream);
// d_out = {a, b} written by a kernel (capturable in a CUDA graph).
cudaError_t set_pair(unsigned long long *d_out, uint64_t a, uint64_t b, cudaStream_t stream);

// ---- K mod p (pg_kmod.cu) ---------------------------------------------------

// For primes base + off[i], i in [d_range[0], d_range[1]) (device values,
// at most max_count of them), at index i - d_range[0]: with walk == nullptr,
// a = K mod p and, when d_b is given, b = R^2 mod p (R = 2^32 or 2^64); with
// a walk, a = the walk step and b = its start residue (all words of the
// primes' width).  Primes below 2^32 use 32-bit words, others 64-bit
// (wide).  K limbs on the device.
// lsb_min_limbs > 0: the least-significant-first chain from that many limbs
// (32-bit primes; 64-bit primes from three quarters of it), else the built-in
// thresholds.  h_klimbs: the same limbs on the host; up to 1024 of them go
// in the launch's parameters instead of shared memory.
cudaError_t kmod_window(const uint32_t *d_klimbs, int nlimbs, uint64_t base, const uint32_t *d_off,
                        const unsigned long long *d_range, uint64_t max_count,
                        const WalkParams *walk, void *d_a, void *d_b, bool wide, cudaStream_t stream,
                        int lsb_min_limbs = 0, const uint32_t *h_klimbs = nullptr);

// Whether K mod p of nlimbs limbs runs least significant limb first, under
// the lsb_min_limbs rule of kmod_window.
bool kmod_lsb(int nlimbs, bool wide, int lsb_min_limbs);

// K's limbs as a kernel parameter (constant bank, read as warp-uniform
// loads): no shared-memory fill and no barrier at the start of every CTA.
constexpr int kParamLimbs = 1024;
template <int N>
struct KLimbs {
    uint32_t limb[N];
};

// K'_g mod p for the G groups of a chain (K'_g = K'_(g-1) * S_g, segment g's
// limbs at d_seg_limbs[d_seg_off[g] .. d_seg_off[g+1]), little-endian) for
// the n primes base + d_off[i]: r_g at d_r[g * n + i], R^2 mod p at
// d_r2[i], words of the primes' width.  nlimbs + G + 1 <= 12288.
// h_seg_limbs / h_seg_off: the same words on the host, passed in the
// launch's parameters when they fit (1024 words).
cudaError_t kmod_chain(const uint32_t *d_seg_limbs, const uint32_t *d_seg_off, int G, int nlimbs, uint64_t base,
                       const uint32_t *d_off, uint64_t n, void *d_r, void *d_r2, bool wide, cudaStream_t stream,
                       const uint32_t *h_seg_limbs = nullptr, const uint32_t *h_seg_off = nullptr);

// K mod q for an explicit list of 32-bit primes (d-primes, tests).
cudaError_t kmod_list32(const uint32_t *d_klimbs, int nlimbs, const uint32_t *d_q, uint32_t n,
                        uint32_t *d_r, cudaStream_t stream);

// ---- large primes (pg_large.cu) -----------------------------------------------

struct JobDev {
    uint64_t mstart;
    uint32_t minc;
    uint32_t sl;        // sieve length
    uint32_t two_sl;    // 2*SL
    uint32_t rows;      // valid m count
    uint32_t half_cols; // H: live columns per side
    uint32_t side_pad;  // Hp: H rounded up to 32, start of the high side
    uint32_t pitch;     // 32-bit words per composite row
    uint32_t *comp;            // rows * pitch words
    uint32_t y_lo;             // walk residues y >= y_lo are offsets X < 0
    WalkParams walk;           // parity-reduced large-prime walk
    uint32_t kmul;             // K = K' * kmul when the walk starts from K' mod p (else 1)
    // tuning: walks of at most direct_steps steps run in the continued
    // fraction's thread, of more than heavy_steps in a CTA of their own, the
    // rest in items of 2^item_shift steps over the CTA
    uint32_t direct_steps, item_shift, heavy_steps;
    // one-job kernel form: bit 0 clear = CTA-pooled items, set = warps alone
    // with a walk list; bits 1 and 2 = K mod p inside the large-prime kernel
    // for windows of 32-bit and of 64-bit primes
    uint32_t large_form;
    // Where a large-prime survivor (row, col) goes.  kMarkComp: OR into comp
    // (method2).  The per-m path (method1) runs the phase twice: kMarkCount
    // counts each row's survivors in row_count, kMarkBucket appends col to
    // the row's bucket at bucket[row_off[row] + k], k from row_count.
    uint32_t mark_mode;
    unsigned long long *row_count;
    const unsigned long long *row_off;
    uint32_t *bucket;
};
constexpr uint32_t kMarkComp = 0, kMarkCount = 1, kMarkBucket = 2;

// The per-m path's rows: each row's large-prime marks from its bucket of
// survivor columns (bucket[row_off[r] .. row_off[r + 1]) for row r, the last
// end in *total) into its comp row, built in shared memory.
cudaError_t bucket_apply(const JobDev &job, const unsigned long long *total, cudaStream_t stream);

struct HeavyPrime;
// Device scratch of the large-prime phase: two counters (group claims, heavy
// primes) and the heavy-prime list.
struct WalkEntry;
struct LargeScratch {
    unsigned long long *counters;  // kLargeCounters words
    HeavyPrime *heavy;
    uint32_t heavy_cap;
    WalkEntry *walks = nullptr;    // walk list of the warp-alone one-job form
    uint32_t walk_cap = 0;
};
constexpr int kLargeCounters = 4;
uint32_t heavy_capacity();
uint32_t walk_capacity();
constexpr size_t kHeavyPrimeBytes = 48;
constexpr size_t kWalkEntryBytes = 32;

// d_mmask: valid-m bitmask over walk indices j (walk.jmax bits), d_ymask:
// live-offset bitmask over walk residues y (walk.w bits), each as {bits, set
// bits before the word} pairs (uint2 per word).
// d_a/d_b as written by kmod_window over the index range d_rrange, which
// contains d_range: with start_in_kernel, K mod p and 2^64 mod p (jobs that
// share K share them; each starts its walk here), else the job's walk step
// and start residue.  With h_klimbs (nlimbs <= kParamLimbs, K's limbs on the
// host), the kernel computes K mod p itself, least significant limb first
// when lsb, and d_a, d_b, d_rrange are not read.
cudaError_t large_window(const JobDev &job, uint64_t base, const uint32_t *d_off,
                         const unsigned long long *d_range, uint64_t max_count, const void *d_a,
                         const void *d_b, const unsigned long long *d_rrange, bool wide,
                         bool start_in_kernel, const uint2 *d_mmask, const uint2 *d_ymask,
                         LargeScratch scratch, cudaStream_t stream, const uint32_t *h_klimbs = nullptr,
                         int nlimbs = 0, bool lsb = true);

// Many jobs in one launch (the batch).  A job: its descriptor (kmul set:
// walks start from K' mod p) and masks; masks_in_shared when they fit the
// launch's dynamic shared memory.
struct LargeJob {
    JobDev job;
    const uint2 *mmask, *ymask;
    int masks_in_shared;
};
// An item: the primes of one job in one prime-table window, in job order;
// tile0 = tiles (kLargeThreads primes) of the items before it.  off, a, b
// point at the item's first prime, its K' mod p (the job's group) and its
// R^2 mod p, all of the primes' width.
struct LargeItem {
    uint32_t job, tile0, count, pad;
    uint64_t base;
    const uint32_t *off;
    const void *a, *b;
};
constexpr uint32_t kLargeTile = 256;
// Both kernels (tiles, then the heavy primes of every job) on one stream;
// smem = the largest job's mask bytes among those with masks_in_shared.
// all_shared: every job's masks fit the launch's shared memory.
cudaError_t large_multi(const LargeJob *d_jobs, const LargeItem *d_items, uint32_t n_items, uint32_t n_tiles,
                        size_t smem, bool wide, LargeScratch scratch, cudaStream_t stream, bool all_shared);

// ---- rows: small primes, merge, extract, format (pg_rows.cu) -----------------

struct RowsDev {
    JobDev job;
    uint32_t x_par;            // parity of the live offsets' index x = X + SL
    uint32_t nb;               // positions x in [0, 2SL] with x % 2 == x_par
    const uint32_t *valid_mi;  // rows entries
    const uint32_t *dist;      // H live distances, ascending
    const uint32_t *live;      // nb bits: the live offsets over (x - x_par) / 2
    // odd primes dividing d (patterns) and their K mod q
    uint32_t nd;
    const uint32_t *dq;
    const uint32_t *dr;
    // odd primes in (P, S1] as offsets from sp_base, and K mod p
    uint32_t sp_base;
    const uint32_t *sp;
    const uint32_t *sr;
    const unsigned long long *sp_range;  // {begin, end} into sp (device)
    uint64_t sp_cap;           // capacity of sr (and of the range)
    uint64_t text_cap;         // capacity of the text buffer
    // outputs
    uint32_t *lists;       // rows * 2H distances (low side then high side)
    uint32_t *counts;      // rows * 2
    uint64_t *row_bytes;   // rows
    int compression;       // 0 plain, 1 RLE
};

// Rows [row_lo, row_hi) (row_lo a multiple of rows_per_block; all by default).
cudaError_t rows_extract(const RowsDev &rd, uint32_t rows_per_block, cudaStream_t stream,
                         uint32_t row_lo = 0, uint32_t row_hi = ~0u);

// Exclusive scan of n 64-bit values, plus *d_base when given; base + total
// written to *d_total.
cudaError_t scan_u64(const uint64_t *d_in, uint64_t *d_out, uint64_t *d_total, uint64_t n,
                     uint64_t *d_tmp, cudaStream_t stream, const uint64_t *d_base = nullptr);
uint64_t scan_tmp_words(uint64_t n);

// Text of rows [row_lo, row_hi) (all by default) at their offsets.
cudaError_t format_rows(const RowsDev &rd, const uint64_t *d_offsets, char *d_text, cudaStream_t stream,
                        uint32_t row_lo = 0, uint32_t row_hi = ~0u);

// ---- C-ABI helpers (pg_tools.cu) -----------------------------------------------

cudaError_t tools_kmod_list64(const uint32_t *d_limbs, int n, const uint64_t *d_q, size_t count,
                              uint64_t *d_out, cudaStream_t stream);
cudaError_t tools_modsearch(const uint64_t *p, const uint64_t *a, const uint64_t *l,
                            const uint64_t *r, uint64_t *k, size_t n, cudaStream_t stream);
cudaError_t tools_large_hits(uint64_t M, uint32_t max_mi, uint32_t sl, uint64_t p, uint64_t r,
                             uint32_t *mi_out, uint64_t *mod_out, size_t cap,
                             unsigned long long *count, cudaStream_t stream);

cudaError_t tools_imad_peak(double *imad_per_s, cudaStream_t stream);

}  // namespace pg
