// K mod p for every sieving prime: a batched multi-limb reduction of
// K = P#/d against 32-bit and 64-bit primes by Montgomery multiplication.
//
// Replaces mpz_fdiv_ui(K, prime) at combined_sieve.cpp:1497 and 1856 (and the
// mpz_mod_ui of 1674).  One thread per prime (four interleaved chains per
// thread for 32-bit primes) reduces K's limbs: most significant first,
// u <- REDC(u * R^2 + limb), for short K; least significant first,
// W <- REDC(W + limb) and one multiply by R^(n+1) mod p at the end, for long
// K, where the cheaper step outweighs the power.  K's limbs sit in shared
// memory and are read as warp-wide broadcasts.
//
// Output, per prime: either r = K mod p and r2 = R^2 mod p (R = 2^32 or 2^64
// by the primes' width), from which a kernel can start any job's walk over
// this K without a division; or, for one job, its walk step and start residue directly
// ((base_r * M + SL) % prime, modulo_search.cpp:345; see WalkParams).
#include "pg_arith.cuh"
#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kKmodThreads = 256;
constexpr int kMaxSharedLimbs = 12288;  // 48 KiB
constexpr int kPrimesPerThread = 4;     // 32-bit primes
constexpr int kLsbMinLimbs = 32;        // 32-bit primes: LSB chain from 32 limbs
constexpr int kLsbMinLimbsWide = 24;    // 64-bit primes: from 12 words

template <bool kWide, bool kLsb>
__global__ void __launch_bounds__(kKmodThreads)
    kmod_kernel(const uint32_t *__restrict__ klimbs, int nlimbs, uint64_t base,
                const uint32_t *__restrict__ off, const unsigned long long *range,
                uint64_t max_count, WalkParams walk, int with_walk, void *a_out, void *b_out) {
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
    // the grid covers max_count primes: one pass of the loop per thread
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (!kWide) {
        // kPrimesPerThread consecutive primes per thread, interleaved chains
        for (uint64_t idx0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kPrimesPerThread; idx0 < n;
             idx0 += stride * kPrimesPerThread) {
            uint32_t p[kPrimesPerThread], r[kPrimesPerThread], pinv[kPrimesPerThread],
                r2[kPrimesPerThread];
#pragma unroll
            for (int k = 0; k < kPrimesPerThread; k++)
                p[k] = idx0 + k < n ? (uint32_t)(base + off[idx0 + k]) : 3u;  // pad with a prime
            if (kLsb)
                kmod32_lsb_multi<kPrimesPerThread>(limbs, nlimbs, p, r, pinv, r2);
            else
                kmod32_multi<kPrimesPerThread>(limbs, nlimbs, p, r, pinv, r2);
#pragma unroll
            for (int k = 0; k < kPrimesPerThread; k++) {
                if (idx0 + k >= n) break;
                uint32_t a = r[k], b = r2[k];
                if (with_walk) walk_start(walk, p[k], r[k], r2[k], a, b, 1, pinv[k]);
                ((uint32_t *)a_out)[idx0 + k] = a;
                if (b_out) ((uint32_t *)b_out)[idx0 + k] = b;
            }
        }
    } else {
        for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
            const uint64_t p = base + off[idx];
            uint64_t pinv, r2;
            const uint64_t r =
                kLsb ? kmod64_lsb(limbs, nlimbs, p, &pinv, &r2) : kmod64(limbs, nlimbs, p, &pinv, &r2);
            uint64_t a = r, b = r2;
            if (with_walk) walk_start(walk, p, r, pinv, r2, a, b);
            ((uint64_t *)a_out)[idx] = a;
            if (b_out) ((uint64_t *)b_out)[idx] = b;
        }
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
                        const WalkParams *walk, void *d_a, void *d_b, bool wide, cudaStream_t stream) {
    if (max_count == 0) return cudaSuccess;
    const WalkParams wp = walk ? *walk : WalkParams{};
    const int ww = walk != nullptr;
    const uint64_t per_thread = wide ? 1 : kPrimesPerThread;
    const uint64_t threads = (max_count + per_thread - 1) / per_thread;
    const unsigned blocks = (unsigned)((threads + kKmodThreads - 1) / kKmodThreads);
    const size_t smem = nlimbs <= kMaxSharedLimbs ? (size_t)nlimbs * sizeof(uint32_t) : 0;
    // least significant limb first once the cheaper step (an add, a multiply
    // and a multiply-add, against a multiply-add, a multiply and a
    // multiply-add) outweighs the R^(n+1) power
    const bool lsb = nlimbs >= (wide ? kLsbMinLimbsWide : kLsbMinLimbs);
    if (wide && lsb)
        kmod_kernel<true, true><<<blocks, kKmodThreads, smem, stream>>>(d_klimbs, nlimbs, base, d_off,
                                                                        d_range, max_count, wp, ww, d_a, d_b);
    else if (wide)
        kmod_kernel<true, false><<<blocks, kKmodThreads, smem, stream>>>(d_klimbs, nlimbs, base, d_off,
                                                                         d_range, max_count, wp, ww, d_a, d_b);
    else if (lsb)
        kmod_kernel<false, true><<<blocks, kKmodThreads, smem, stream>>>(d_klimbs, nlimbs, base, d_off,
                                                                         d_range, max_count, wp, ww, d_a, d_b);
    else
        kmod_kernel<false, false><<<blocks, kKmodThreads, smem, stream>>>(d_klimbs, nlimbs, base, d_off,
                                                                          d_range, max_count, wp, ww, d_a, d_b);
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
