// Large-prime phase: for every prime p > 4*SL+2, every m in
// [mstart, mstart+minc) and offset X in [-SL, SL] with p | m*K + X.
//
// Replaces method2_large_primes (combined_sieve.cpp:1763-2011) and the
// enumeration modulo_search_euclid_all_large (modulo_search.cpp:339-376).
// With y(mi) = (r*(mstart+mi) + SL) mod p, r = K mod p, a hit is y <= 2*SL and
// marks offset X = SL - y of m = mstart + mi.
//
// The reference runs one Euclid modulo search per hit.  Here one search finds
// the first hit of a range of mi, then Slater's three-gap theorem gives each
// following hit in O(1): the return time of y -> y + r (mod p) to [0, 2*SL]
// takes only the values kp, kn, kp+kn, decided by comparing y against the two
// record residues up and dn (pg::three_gap).
//
// Work is balanced by splitting each prime's mi range into chunks with about
// `hits_per_item` expected hits; a CTA takes 256 primes, expands their chunks
// and lets its threads pull (prime, chunk) items.  Hits on a valid m and a
// live offset set one bit of the L2-resident composite bitset with a global
// atomicOr.
#include "pg_arith.cuh"
#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kLargeThreads = 256;

struct MarkHit {
    const JobDev &job;
    __device__ __forceinline__ void operator()(uint64_t mi, uint64_t y) const {
        if (y > job.two_sl || mi >= job.minc) return;  // unreachable for prime moduli
        const uint32_t x = job.two_sl - (uint32_t)y;
        const int32_t row = __ldg(&job.row_of_mi[mi]);
        if (row < 0) return;
        const int32_t col = __ldg(&job.col_of_x[x]);
        if (col < 0) return;
        atomicOr(&job.comp[(uint64_t)row * job.pitch + ((uint32_t)col >> 5)], 1u << (col & 31));
    }
};

template <typename T>
__global__ void __launch_bounds__(kLargeThreads)
    large_kernel(JobDev job, uint64_t base, const uint32_t *__restrict__ off,
                 const unsigned long long *count, uint64_t max_count, const T *__restrict__ r_in,
                 const T *__restrict__ t0_in, uint32_t hits_per_item) {
    __shared__ uint32_t s_start[kLargeThreads + 1];
    __shared__ T s_p[kLargeThreads], s_r[kLargeThreads], s_t0[kLargeThreads];
    __shared__ uint32_t s_len[kLargeThreads];
    const uint64_t n = min((uint64_t)*count, max_count);
    const uint64_t first = (uint64_t)blockIdx.x * kLargeThreads;
    if (first >= n) return;
    const uint64_t i = first + threadIdx.x;
    uint32_t nch = 0;
    if (i < n) {
        const T p = (T)(base + off[i]);
        s_p[threadIdx.x] = p;
        s_r[threadIdx.x] = r_in[i];
        s_t0[threadIdx.x] = t0_in[i];
        const float e = (float)job.minc * (float)(job.two_sl + 1) / (float)p;
        float want = ceilf(e / (float)hits_per_item);
        uint32_t c = want < 1.f ? 1u : (want > (float)job.minc ? job.minc : (uint32_t)want);
        uint32_t len = (job.minc + c - 1) / c;
        nch = (job.minc + len - 1) / len;
        s_len[threadIdx.x] = len;
    }
    s_start[threadIdx.x + 1] = nch;
    if (threadIdx.x == 0) s_start[0] = 0;
    __syncthreads();
    // inclusive scan over s_start[1..256]
    for (int o = 1; o < kLargeThreads; o <<= 1) {
        uint32_t v = threadIdx.x >= (uint32_t)o ? s_start[threadIdx.x + 1 - o] : 0;
        __syncthreads();
        s_start[threadIdx.x + 1] += v;
        __syncthreads();
    }
    const uint32_t total = s_start[kLargeThreads];
    for (uint32_t it = threadIdx.x; it < total; it += kLargeThreads) {
        // slot s with s_start[s] <= it < s_start[s+1]
        uint32_t lo = 0, hi = kLargeThreads;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (s_start[mid] <= it) lo = mid;
            else hi = mid;
        }
        const uint32_t s = lo;
        const uint32_t c = it - s_start[s];
        const uint64_t mi_lo = (uint64_t)c * s_len[s];
        uint64_t mi_hi = mi_lo + s_len[s];
        if (mi_hi > job.minc) mi_hi = job.minc;
        const T p = s_p[s], r = s_r[s];
        const T y = advance_residue(s_t0[s], mi_lo, r, p);
        MarkHit mark{job};
        enumerate_hits<T>(p, r, y, mi_lo, mi_hi, (T)job.two_sl, mark);
    }
}

}  // namespace

cudaError_t large_window(const JobDev &job, uint64_t base, const uint32_t *d_off,
                         const unsigned long long *d_count, uint64_t max_count, const void *d_r,
                         const void *d_t0, bool wide, uint32_t hits_per_item, cudaStream_t stream) {
    if (max_count == 0) return cudaSuccess;
    uint64_t blocks = (max_count + kLargeThreads - 1) / kLargeThreads;
    if (wide)
        large_kernel<uint64_t><<<(unsigned)blocks, kLargeThreads, 0, stream>>>(
            job, base, d_off, d_count, max_count, (const uint64_t *)d_r, (const uint64_t *)d_t0, hits_per_item);
    else
        large_kernel<uint32_t><<<(unsigned)blocks, kLargeThreads, 0, stream>>>(
            job, base, d_off, d_count, max_count, (const uint32_t *)d_r, (const uint32_t *)d_t0, hits_per_item);
    return cudaGetLastError();
}

}  // namespace pg
