// Prime generation: a segmented sieve of Eratosthenes over odd numbers.
//
// Replaces the reference's primesieve::iterator loops
// (combined_sieve.cpp:1475-1502, 1662-1668, 1851-1852): every prime below
// the sieve limit is produced on the device and stays resident in HBM.
//
// One CTA sieves one segment of kSegBits odd numbers in a 32 KiB shared
// bitmap (bit set = composite):
//   * base primes below 64 stamp a precomputed 32-bit pattern into every word;
//   * base primes in [64, 2048) are marked warp-cooperatively;
//   * larger base primes are marked one per thread;
// then the block compacts its primes (offsets from the window start) into a
// global list with one atomicAdd per block.  The list is unordered: every
// consumer treats primes independently.
#include "pg_internal.h"

#include <algorithm>
#include <cmath>

namespace pg {

namespace {

constexpr int kSieveThreads = 512;
constexpr uint32_t kSegWords = kSegBits / 32;
constexpr int kTinyCount = 17;

// The odd primes below 64, as compile-time constants (the loops over them
// are unrolled, so every division by one becomes a multiply and shift).
__host__ __device__ constexpr uint32_t tiny_q(int t) {
    constexpr uint32_t q[kTinyCount] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61};
    return q[t];
}

// bits at multiples of q inside a 32-bit word (q >= 32 -> bit 0 only)
__host__ __device__ constexpr uint32_t tiny_pattern(uint32_t q) {
    uint32_t m = 0;
    for (uint32_t b = 0; b < 32; b += q) m |= 1u << b;
    return m;
}

// number of base primes q with q*q <= hi (base ascending)
__device__ uint32_t base_bound(const uint32_t *base, uint32_t nbase, uint64_t hi) {
    uint32_t lo = 0, up = nbase;
    while (lo < up) {
        uint32_t mid = (lo + up) >> 1;
        uint64_t q = base[mid];
        if (q * q <= hi) lo = mid + 1;
        else up = mid;
    }
    return lo;
}

// Bit index (odd numbers from seg_lo, odd) of the first odd multiple of q at
// or above max(q^2, seg_lo), for q^2 <= seg_hi: below 2q + 2^18, so 32 bits.
// With rem = seg_lo mod q and d = (q - rem) mod q, seg_lo + d is the first
// multiple, odd iff d is even (seg_lo odd); else the next odd one is q on.
// Segments below 2^32 take a 32-bit remainder.
__device__ __forceinline__ uint32_t first_index(uint32_t q, uint64_t seg_lo, bool lo32) {
    const uint64_t sq = (uint64_t)q * q;
    if (sq >= seg_lo) return (uint32_t)((sq - seg_lo) >> 1);
    const uint32_t rem = lo32 ? (uint32_t)seg_lo % q : (uint32_t)(seg_lo % q);
    const uint32_t d = rem == 0 ? 0u : q - rem;
    return (d & 1u) ? (d + q) >> 1 : d >> 1;
}

// Marks composites of the segment [seg_lo, seg_hi] (seg_lo odd) in `bits`.
// Primes themselves stay clear; 1 is marked.  Blocks of kSieveThreads.
__device__ void sieve_segment(uint32_t *bits, uint64_t seg_lo, uint64_t seg_hi,
                              const uint32_t *base, uint32_t nbase) {
    const uint32_t nbits = (uint32_t)((seg_hi - seg_lo) / 2 + 1);
    __shared__ uint32_t s_nq;
    if (threadIdx.x == 0) s_nq = base_bound(base, nbase, seg_hi);

    // tiny primes: per-word patterns; this also initialises every word.
    // Word w holds indices 32w + b; q divides seg_lo + 2(32w + b) for
    // b = o (mod q), o = j0 - 32w mod q with j0 = -seg_lo (q+1)/2 mod q.
    // Each thread's words are kSieveThreads apart, so o drops by a constant.
    uint32_t o[kTinyCount];
#pragma unroll
    for (int t = 0; t < kTinyCount; t++) {
        const uint32_t q = tiny_q(t);
        const uint32_t neg = (q - (uint32_t)(seg_lo % q)) % q;
        const uint32_t j0 = neg * ((q + 1) / 2) % q;
        o[t] = (j0 + q - (32u * threadIdx.x) % q) % q;
    }
    constexpr uint32_t wstep = 32u * kSieveThreads;
    for (uint32_t w = threadIdx.x; w < kSegWords; w += kSieveThreads) {
        uint32_t word = 0;
#pragma unroll
        for (int t = 0; t < kTinyCount; t++) {
            const uint32_t q = tiny_q(t);
            if (q < 32) word |= tiny_pattern(q) << o[t];
            else if (o[t] < 32) word |= 1u << o[t];
            const uint32_t d = wstep % q;
            o[t] = o[t] >= d ? o[t] - d : o[t] + q - d;
        }
        bits[w] = word;
    }
    __syncthreads();
    if (threadIdx.x == 0 && seg_lo <= tiny_q(kTinyCount - 1)) {
        // the tiny primes themselves are prime
#pragma unroll
        for (int t = 0; t < kTinyCount; t++) {
            const uint64_t q = tiny_q(t);
            if (q >= seg_lo && q <= seg_hi) {
                const uint32_t j = (uint32_t)((q - seg_lo) / 2);
                bits[j >> 5] &= ~(1u << (j & 31));
            }
        }
    }
    if (threadIdx.x == 0 && seg_lo == 1) atomicOr(&bits[0], 1u);  // 1 is not prime
    __syncthreads();

    const uint32_t nq = s_nq;
    // base primes are odd primes starting at 3; skip those below 64 (index of
    // first prime >= 64 is 17, since 3..61 are the 17 odd primes below 64)
    const uint32_t first_mid = 17;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const bool lo32 = seg_hi <= 0xFFFFFFFFull;
    // medium primes: one warp per prime
    for (uint32_t i = first_mid + warp; i < nq; i += nwarps) {
        const uint32_t q = base[i];
        if (q >= 2048) break;
        for (uint32_t j = first_index(q, seg_lo, lo32) + lane * q; j < nbits; j += 32 * q)
            atomicOr(&bits[j >> 5], 1u << (j & 31));
    }
    // large primes: one thread per prime
    uint32_t first_large = first_mid;
    {
        // index of first base prime >= 2048 (binary search, cheap)
        uint32_t lo = first_mid, up = nq;
        while (lo < up) {
            uint32_t mid = (lo + up) >> 1;
            if (base[mid] < 2048) lo = mid + 1;
            else up = mid;
        }
        first_large = lo;
    }
    for (uint32_t i = first_large + threadIdx.x; i < nq; i += blockDim.x) {
        const uint32_t q = base[i];
        for (uint32_t j = first_index(q, seg_lo, lo32); j < nbits; j += q)
            atomicOr(&bits[j >> 5], 1u << (j & 31));
    }
    __syncthreads();
}

// Unordered compaction of a window's primes (offsets from win_lo).  Each
// warp owns kSegWords / 16 consecutive words and writes their primes in
// rounds of 32 words, one word per lane: a round's primes are contiguous in
// the output, so its stores touch a few cache lines rather than one per lane.
__global__ void __launch_bounds__(kSieveThreads)
    sieve_window_kernel(uint64_t win_lo, uint64_t win_hi, uint64_t first_odd, const uint32_t *base,
                        uint32_t nbase, uint32_t *out, uint64_t cap,
                        unsigned long long *count) {
    constexpr uint32_t kWarps = kSieveThreads / 32, kWarpWords = kSegWords / kWarps;
    __shared__ uint32_t bits[kSegWords];
    __shared__ uint32_t s_warp[kWarps];
    __shared__ unsigned long long s_base;
    const uint64_t seg_lo = first_odd + (uint64_t)blockIdx.x * kSegSpan;
    if (seg_lo > win_hi) return;
    uint64_t seg_hi = seg_lo + kSegSpan - 2;
    if (seg_hi > win_hi) seg_hi = win_hi;
    sieve_segment(bits, seg_lo, seg_hi, base, nbase);

    const uint32_t nbits = (uint32_t)((seg_hi - seg_lo) / 2 + 1);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t wbeg = warp * kWarpWords;
    // primes (clear bits below nbits) of word w
    auto primes_of = [&](uint32_t w) -> uint32_t {
        const uint32_t b0 = w * 32;
        if (b0 >= nbits) return 0u;
        const uint32_t valid = (nbits - b0 >= 32) ? 0xFFFFFFFFu : ((1u << (nbits - b0)) - 1);
        return ~bits[w] & valid;
    };
    uint32_t cnt = 0;
    for (uint32_t w = wbeg + lane; w < wbeg + kWarpWords; w += 32) cnt += __popc(primes_of(w));
    cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if (lane == 0) s_warp[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (uint32_t k = 0; k < kWarps; k++) {
            const uint32_t c = s_warp[k];
            s_warp[k] = total;
            total += c;
        }
        s_base = atomicAdd(count, (unsigned long long)total);
    }
    __syncthreads();
    uint64_t pos = s_base + s_warp[warp];
    for (uint32_t w = wbeg + lane; w < wbeg + kWarpWords; w += 32) {
        uint32_t primes = primes_of(w);
        const uint32_t c = __popc(primes);
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        uint64_t at = pos + incl - c;
        while (primes) {
            const uint32_t b = __ffs(primes) - 1;
            primes &= primes - 1;
            const uint64_t v = seg_lo + 2ull * (w * 32 + b);
            if (at < cap) out[at] = (uint32_t)(v - win_lo);
            at++;
        }
        pos += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
}

// Ordered sieve of [3, hi] for base primes: bitmaps + per-segment counts.
__global__ void __launch_bounds__(kSieveThreads)
    sieve_bitmap_kernel(uint64_t hi, const uint32_t *base, uint32_t nbase, uint32_t *gbits,
                        uint32_t *seg_counts) {
    __shared__ uint32_t bits[kSegWords];
    const uint64_t seg_lo = 1 + (uint64_t)blockIdx.x * kSegSpan;
    uint64_t seg_hi = seg_lo + kSegSpan - 2;
    if (seg_hi > hi) seg_hi = hi;
    sieve_segment(bits, seg_lo, seg_hi, base, nbase);
    const uint32_t nbits = (uint32_t)((seg_hi - seg_lo) / 2 + 1);
    uint32_t cnt = 0;
    for (uint32_t w = threadIdx.x; w < kSegWords; w += blockDim.x) {
        uint32_t b0 = w * 32;
        uint32_t valid = 0;
        if (b0 < nbits) valid = (nbits - b0 >= 32) ? 0xFFFFFFFFu : ((1u << (nbits - b0)) - 1);
        uint32_t primes = ~bits[w] & valid;
        gbits[(uint64_t)blockIdx.x * kSegWords + w] = primes;
        cnt += __popc(primes);
    }
    cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if ((threadIdx.x & 31) == 0) atomicAdd(&seg_counts[blockIdx.x], cnt);
}

// Single CTA: ordered extraction of primes from bitmaps (values 1 + 2j).
__global__ void __launch_bounds__(1024) ordered_extract_kernel(const uint32_t *gbits, uint64_t nwords,
                                                               uint32_t *out, uint32_t *count) {
    __shared__ uint32_t s_scan[1024];
    __shared__ uint32_t s_total;
    if (threadIdx.x == 0) s_total = 0;
    __syncthreads();
    for (uint64_t w0 = 0; w0 < nwords; w0 += 1024) {
        uint64_t w = w0 + threadIdx.x;
        uint32_t word = w < nwords ? gbits[w] : 0;
        uint32_t c = __popc(word);
        s_scan[threadIdx.x] = c;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            uint32_t v = threadIdx.x >= (uint32_t)off ? s_scan[threadIdx.x - off] : 0;
            __syncthreads();
            s_scan[threadIdx.x] += v;
            __syncthreads();
        }
        uint32_t pos = s_total + s_scan[threadIdx.x] - c;
        // segment s, word k: values 1 + 2*(s*kSegBits + 32k + b) = 1 + 2*(32w + b)
        while (word) {
            uint32_t b = __ffs(word) - 1;
            word &= word - 1;
            out[pos++] = (uint32_t)(1 + 2 * (32 * w + b));
        }
        __syncthreads();
        if (threadIdx.x == 1023) s_total += s_scan[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = s_total;
}

// Odd primes below 2^16 by trial division against odd primes below 256.
__global__ void __launch_bounds__(1024) small_primes_kernel(uint32_t *out, uint32_t *count) {
    __shared__ uint32_t s_scan[1024];
    __shared__ uint32_t s_total;
    if (threadIdx.x == 0) s_total = 0;
    __syncthreads();
    for (uint32_t v0 = 3; v0 < 65536; v0 += 2048) {
        uint32_t v = v0 + 2 * threadIdx.x;
        bool prime = v < 65536;
        for (uint32_t d = 3; prime && d * d <= v; d += 2)
            if (v % d == 0) prime = false;
        s_scan[threadIdx.x] = prime;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            uint32_t x = threadIdx.x >= (uint32_t)off ? s_scan[threadIdx.x - off] : 0;
            __syncthreads();
            s_scan[threadIdx.x] += x;
            __syncthreads();
        }
        if (prime) out[s_total + s_scan[threadIdx.x] - 1] = v;
        __syncthreads();
        if (threadIdx.x == 1023) s_total += s_scan[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = s_total;
}

// Sorted sieve, pass 1: bitmap of primes and count per segment.
__global__ void __launch_bounds__(kSieveThreads)
    seg_bitmap_kernel(uint64_t win_hi, uint64_t first_odd, const uint32_t *base, uint32_t nbase,
                      uint32_t *gbits, uint64_t *seg_counts) {
    __shared__ uint32_t bits[kSegWords];
    __shared__ uint32_t s_cnt;
    const uint64_t seg_lo = first_odd + (uint64_t)blockIdx.x * kSegSpan;
    uint64_t seg_hi = seg_lo + kSegSpan - 2;
    if (seg_hi > win_hi) seg_hi = win_hi;
    if (threadIdx.x == 0) s_cnt = 0;
    sieve_segment(bits, seg_lo, seg_hi, base, nbase);
    const uint32_t nbits = (uint32_t)((seg_hi - seg_lo) / 2 + 1);
    uint32_t cnt = 0;
    for (uint32_t w = threadIdx.x; w < kSegWords; w += blockDim.x) {
        const uint32_t b0 = w * 32;
        uint32_t valid = 0;
        if (b0 < nbits) valid = (nbits - b0 >= 32) ? 0xFFFFFFFFu : ((1u << (nbits - b0)) - 1);
        const uint32_t primes = ~bits[w] & valid;
        gbits[(uint64_t)blockIdx.x * kSegWords + w] = primes;
        cnt += __popc(primes);
    }
    cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s_cnt, cnt);
    __syncthreads();
    if (threadIdx.x == 0) seg_counts[blockIdx.x] = s_cnt;
}

// Sorted sieve, pass 2: each segment writes its primes (offsets from win_lo)
// at its prefix-sum position, in increasing order.
__global__ void __launch_bounds__(kSieveThreads)
    seg_extract_kernel(uint64_t win_lo, uint64_t first_odd, const uint32_t *gbits,
                       const uint64_t *seg_offsets, uint32_t *out, uint64_t cap) {
    __shared__ uint32_t s_scan[kSieveThreads];
    const uint64_t seg_lo = first_odd + (uint64_t)blockIdx.x * kSegSpan;
    const uint32_t per = kSegWords / kSieveThreads;
    const uint32_t *g = gbits + (uint64_t)blockIdx.x * kSegWords + threadIdx.x * per;
    uint32_t words[kSegWords / kSieveThreads];
    uint32_t cnt = 0;
#pragma unroll
    for (uint32_t k = 0; k < per; k++) {
        words[k] = g[k];
        cnt += __popc(words[k]);
    }
    s_scan[threadIdx.x] = cnt;
    __syncthreads();
    for (int off = 1; off < kSieveThreads; off <<= 1) {
        uint32_t v = threadIdx.x >= (uint32_t)off ? s_scan[threadIdx.x - off] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += v;
        __syncthreads();
    }
    uint64_t pos = seg_offsets[blockIdx.x] + s_scan[threadIdx.x] - cnt;
#pragma unroll
    for (uint32_t k = 0; k < per; k++) {
        uint32_t m = words[k];
        const uint32_t b0 = (threadIdx.x * per + k) * 32;
        while (m) {
            const uint32_t b = __ffs(m) - 1;
            m &= m - 1;
            if (pos < cap) out[pos] = (uint32_t)(seg_lo + 2ull * (b0 + b) - win_lo);
            pos++;
        }
    }
}

// [begin, end) of the sorted list base + off[0..count) within [lo_val, hi_val].
__global__ void range_kernel(const uint32_t *off, uint64_t count, uint64_t base, uint64_t lo_val,
                             uint64_t hi_val, unsigned long long *out) {
    if (threadIdx.x != 0) return;
    uint64_t a = 0, b = count;
    while (a < b) {  // first >= lo_val
        uint64_t mid = (a + b) >> 1;
        if (base + off[mid] < lo_val) a = mid + 1;
        else b = mid;
    }
    uint64_t c = a, d = count;
    while (c < d) {  // first > hi_val
        uint64_t mid = (c + d) >> 1;
        if (base + off[mid] <= hi_val) c = mid + 1;
        else d = mid;
    }
    out[0] = a;
    out[1] = hi_val >= lo_val ? c : a;
}

__global__ void set_pair_kernel(unsigned long long *out, unsigned long long a, unsigned long long b) {
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = b;
    }
}

uint64_t isqrt64(uint64_t n) {
    uint64_t r = (uint64_t)std::sqrt((double)n);
    while (r * r > n) r--;
    while ((r + 1) * (r + 1) <= n) r++;
    return r;
}

}  // namespace

uint64_t prime_count_bound(uint64_t lo, uint64_t hi) {
    if (hi < lo) return 0;
    double y = (double)(hi - lo + 1);
    if (y < 1e4) return (uint64_t)y / 2 + 64;
    // pi(x + y) - pi(x) <= 2y / ln y  (Montgomery & Vaughan, 1973)
    return (uint64_t)(2.0 * y / std::log(y)) + 1024;
}

cudaError_t base_primes_build(BasePrimes &bp, uint64_t limit, cudaStream_t stream) {
    uint64_t need = isqrt64(limit) + 1;
    if (bp.d_primes && bp.covers >= limit) return cudaSuccess;
    base_primes_free(bp);
    cudaError_t e;
    // level 0: odd primes < 2^16
    uint32_t *d_small = nullptr, *d_cnt = nullptr;
    const uint32_t small_cap = 6600;
    if ((e = cudaMalloc(&d_small, small_cap * sizeof(uint32_t)))) return e;
    if ((e = cudaMalloc(&d_cnt, 2 * sizeof(uint32_t)))) return e;
    small_primes_kernel<<<1, 1024, 0, stream>>>(d_small, d_cnt);
    uint32_t nsmall = 0;
    if ((e = cudaMemcpyAsync(&nsmall, d_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream))) return e;
    if ((e = cudaStreamSynchronize(stream))) return e;
    if (need < 65536) {
        bp.d_primes = d_small;
        bp.count = nsmall;
        bp.covers = 65535ull * 65535ull;
        cudaFree(d_cnt);
        return cudaSuccess;
    }
    // level 1: odd primes in [3, need] from bitmaps sieved by level 0
    uint64_t nseg = (need - 1) / kSegSpan + 1;
    uint32_t *d_bits = nullptr, *d_segc = nullptr, *d_out = nullptr;
    uint64_t cap = prime_count_bound(1, need) + 16;
    if ((e = cudaMalloc(&d_bits, nseg * kSegWords * sizeof(uint32_t)))) return e;
    if ((e = cudaMalloc(&d_segc, nseg * sizeof(uint32_t)))) return e;
    if ((e = cudaMalloc(&d_out, cap * sizeof(uint32_t)))) return e;
    cudaMemsetAsync(d_segc, 0, nseg * sizeof(uint32_t), stream);
    sieve_bitmap_kernel<<<(unsigned)nseg, kSieveThreads, 0, stream>>>(need, d_small, nsmall, d_bits,
                                                                      d_segc);
    ordered_extract_kernel<<<1, 1024, 0, stream>>>(d_bits, nseg * kSegWords, d_out, d_cnt + 1);
    uint32_t nout = 0;
    if ((e = cudaMemcpyAsync(&nout, d_cnt + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream))) return e;
    if ((e = cudaStreamSynchronize(stream))) return e;
    if ((e = cudaGetLastError())) return e;
    cudaFree(d_bits);
    cudaFree(d_segc);
    cudaFree(d_small);
    cudaFree(d_cnt);
    bp.d_primes = d_out;
    bp.count = nout;
    bp.covers = need * need - 1;
    return cudaSuccess;
}

void base_primes_free(BasePrimes &bp) {
    if (bp.d_primes) cudaFree(bp.d_primes);
    bp = BasePrimes{};
}

cudaError_t sieve_window(const BasePrimes &bp, uint64_t lo, uint64_t hi, uint32_t *d_out,
                         uint64_t cap, unsigned long long *d_count, cudaStream_t stream) {
    if (hi < lo) return cudaSuccess;
    if (hi > bp.covers) return cudaErrorInvalidValue;
    if (hi - lo >= (1ull << 32)) return cudaErrorInvalidValue;
    uint64_t first_odd = lo | 1;
    if (first_odd < 3) first_odd = 3;
    if (first_odd > hi) return cudaSuccess;
    uint64_t nseg = (hi - first_odd) / kSegSpan + 1;
    sieve_window_kernel<<<(unsigned)nseg, kSieveThreads, 0, stream>>>(
        lo, hi, first_odd, bp.d_primes, bp.count, d_out, cap, d_count);
    return cudaGetLastError();
}

uint64_t sieve_sorted_tmp_bytes(uint64_t lo, uint64_t hi) {
    uint64_t first_odd = std::max<uint64_t>(lo | 1, 3);
    if (first_odd > hi) return 256;
    uint64_t nseg = (hi - first_odd) / kSegSpan + 1;
    return nseg * kSegWords * 4 + nseg * 16 + scan_tmp_words(nseg) * 8 + 256;
}

cudaError_t sieve_window_sorted(const BasePrimes &bp, uint64_t lo, uint64_t hi, uint32_t *d_out,
                                uint64_t cap, unsigned long long *d_count, void *d_tmp,
                                cudaStream_t stream) {
    if (hi > bp.covers || hi - lo >= (1ull << 32)) return cudaErrorInvalidValue;
    uint64_t first_odd = std::max<uint64_t>(lo | 1, 3);
    if (first_odd > hi) return cudaMemsetAsync(d_count, 0, 8, stream);
    const uint64_t nseg = (hi - first_odd) / kSegSpan + 1;
    uint32_t *gbits = (uint32_t *)d_tmp;
    uint64_t *seg_counts = (uint64_t *)(gbits + nseg * kSegWords);
    uint64_t *seg_offsets = seg_counts + nseg;
    uint64_t *scan_tmp = seg_offsets + nseg;
    seg_bitmap_kernel<<<(unsigned)nseg, kSieveThreads, 0, stream>>>(hi, first_odd, bp.d_primes,
                                                                    bp.count, gbits, seg_counts);
    cudaError_t e = scan_u64(seg_counts, seg_offsets, (uint64_t *)d_count, nseg, scan_tmp, stream);
    if (e) return e;
    seg_extract_kernel<<<(unsigned)nseg, kSieveThreads, 0, stream>>>(lo, first_odd, gbits,
                                                                     seg_offsets, d_out, cap);
    return cudaGetLastError();
}

cudaError_t find_range(const uint32_t *d_off, uint64_t count, uint64_t base, uint64_t lo_val,
                       uint64_t hi_val, unsigned long long *d_out, cudaStream_t stream) {
    range_kernel<<<1, 32, 0, stream>>>(d_off, count, base, lo_val, hi_val, d_out);
    return cudaGetLastError();
}

cudaError_t set_pair(unsigned long long *d_out, uint64_t a, uint64_t b, cudaStream_t stream) {
    set_pair_kernel<<<1, 32, 0, stream>>>(d_out, a, b);
    return cudaGetLastError();
}

}  // namespace pg
