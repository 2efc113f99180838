// K mod p for every sieving prime: a batched multi-limb reduction of
// K = P#/d against 32-bit and 64-bit primes by Montgomery multiplication.
//
// Replaces mpz_fdiv_ui(K, prime) at combined_sieve.cpp:1497 and 1856 (and the
// mpz_mod_ui of 1674).  One thread per prime walks the limbs of K from the
// most significant end: u <- REDC(u * R^2 + limb), so after the last limb
// u = K * R^-1 and REDC(u * R^2) = K mod p.  K's limbs sit in shared memory
// and are read as warp-wide broadcasts.
//
// Each prime also gets t0 = (r * mstart + SL) mod p, the starting residue of
// the large-prime walk ((base_r * M + SL) % prime, modulo_search.cpp:345).
#include "pg_arith.cuh"
#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kKmodThreads = 256;
constexpr int kMaxSharedLimbs = 12288;  // 48 KiB
constexpr int kPrimesPerThread = 4;     // 32-bit primes

template <bool kWide>
__global__ void __launch_bounds__(kKmodThreads)
    kmod_kernel(const uint32_t *__restrict__ klimbs, int nlimbs, uint64_t base,
                const uint32_t *__restrict__ off, const unsigned long long *range,
                uint64_t max_count, WalkParams walk, int with_walk, void *r_out, void *t0_out) {
    extern __shared__ uint32_t s_limbs[];
    const bool in_shared = nlimbs <= kMaxSharedLimbs;
    if (in_shared)
        for (int i = threadIdx.x; i < nlimbs; i += blockDim.x) s_limbs[i] = klimbs[i];
    __syncthreads();
    const uint32_t *limbs = in_shared ? s_limbs : klimbs;
    // primes off[range[0] .. range[1]), never more than the list's capacity
    const uint64_t begin = range[0];
    const uint64_t n = min((uint64_t)(range[1] - begin), max_count);
    off += begin;
    if (!kWide) {
        // kPrimesPerThread consecutive primes per thread, interleaved chains
        const uint64_t idx0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kPrimesPerThread;
        if (idx0 >= n) return;
        uint32_t p[kPrimesPerThread], r[kPrimesPerThread], pinv[kPrimesPerThread],
            r2[kPrimesPerThread];
#pragma unroll
        for (int k = 0; k < kPrimesPerThread; k++)
            p[k] = idx0 + k < n ? (uint32_t)(base + off[idx0 + k]) : 3u;  // pad with a prime
        kmod32_multi<kPrimesPerThread>(limbs, nlimbs, p, r, pinv, r2);
#pragma unroll
        for (int k = 0; k < kPrimesPerThread; k++) {
            if (idx0 + k >= n) break;
            if (!with_walk) {
                ((uint32_t *)r_out)[idx0 + k] = r[k];
                continue;
            }
            const uint32_t rh = half_mod(r[k], p[k]);
            const uint32_t c = walk.c_add + (walk.odd_d ? (p[k] >> 1) + 1 : 0u);
            ((uint32_t *)r_out)[idx0 + k] = walk.odd_d ? rh : r[k];
            ((uint32_t *)t0_out)[idx0 + k] = start32(rh, walk.m0, c, p[k], pinv[k], r2[k]);
        }
    } else {
        const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (idx >= n) return;
        const uint64_t p = base + off[idx];
        const uint64_t r = kmod64(limbs, nlimbs, p);
        if (!with_walk) {
            ((uint64_t *)r_out)[idx] = r;
            return;
        }
        const uint64_t rh = half_mod(r, p);
        const uint64_t c = walk.c_add + (walk.odd_d ? (p >> 1) + 1 : 0ull);
        uint64_t t = mulmod_u64(rh, walk.m0 % p, p, 1.0 / (double)p) + c;
        if (t >= p) t -= p;
        ((uint64_t *)r_out)[idx] = walk.odd_d ? rh : r;
        ((uint64_t *)t0_out)[idx] = t;
    }
}

__global__ void __launch_bounds__(kKmodThreads)
    kmod_list_kernel(const uint32_t *__restrict__ klimbs, int nlimbs, const uint32_t *q, uint32_t n,
                     uint32_t *r) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t pinv, r2;
    r[i] = kmod32(klimbs, nlimbs, q[i], pinv, r2);
}

}  // namespace

cudaError_t kmod_window(const uint32_t *d_klimbs, int nlimbs, uint64_t base, const uint32_t *d_off,
                        const unsigned long long *d_range, uint64_t max_count,
                        const WalkParams *walk, void *d_r, void *d_t0, bool wide,
                        cudaStream_t stream) {
    const WalkParams wp = walk ? *walk : WalkParams{};
    const int with_walk = walk != nullptr;
    if (max_count == 0) return cudaSuccess;
    const uint64_t per_thread = wide ? 1 : kPrimesPerThread;
    const uint64_t threads = (max_count + per_thread - 1) / per_thread;
    uint64_t blocks = (threads + kKmodThreads - 1) / kKmodThreads;
    size_t smem = nlimbs <= kMaxSharedLimbs ? (size_t)nlimbs * sizeof(uint32_t) : 0;
    if (wide)
        kmod_kernel<true><<<(unsigned)blocks, kKmodThreads, smem, stream>>>(
            d_klimbs, nlimbs, base, d_off, d_range, max_count, wp, with_walk, d_r, d_t0);
    else
        kmod_kernel<false><<<(unsigned)blocks, kKmodThreads, smem, stream>>>(
            d_klimbs, nlimbs, base, d_off, d_range, max_count, wp, with_walk, d_r, d_t0);
    return cudaGetLastError();
}

cudaError_t kmod_list32(const uint32_t *d_klimbs, int nlimbs, const uint32_t *d_q, uint32_t n,
                        uint32_t *d_r, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    kmod_list_kernel<<<(n + kKmodThreads - 1) / kKmodThreads, kKmodThreads, 0, stream>>>(
        d_klimbs, nlimbs, d_q, n, d_r);
    return cudaGetLastError();
}

}  // namespace pg
