// K mod p for every sieving prime: a batched multi-limb reduction of
// K = P#/d against 32-bit and 64-bit primes by Montgomery multiplication.
//
// Replaces mpz_fdiv_ui(K, prime) at combined_sieve.cpp:1497 and 1856 (and the
// mpz_mod_ui of 1674).  One thread per prime (eight interleaved chains per
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
#include <algorithm>
#include <cstring>

#include "pg_arith.cuh"
#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kKmodThreads = 256;
constexpr int kMaxSharedLimbs = 12288;  // 48 KiB
constexpr int kPrimesPerThread = 8;     // 32-bit primes
constexpr int kChainPrimesPerThread = 4;  // 32-bit primes of the chained K' mod p (batch)
constexpr int kLsbMinLimbs = 32;        // 32-bit primes: LSB chain from 32 limbs
constexpr int kLsbMinLimbsWide = 24;    // 64-bit primes: from 12 words

// kParam: K's limbs come in `kl` (nlimbs <= kParamLimbs); otherwise they are
// copied from klimbs to shared memory (or read from global when too long).
template <bool kWide, bool kLsb, bool kParam>
__global__ void __launch_bounds__(kKmodThreads)
    kmod_kernel(const __grid_constant__ KLimbs<kParam ? kParamLimbs : 1> kl, const uint32_t *__restrict__ klimbs,
                int nlimbs, uint64_t base, const uint32_t *__restrict__ off, const unsigned long long *range,
                uint64_t max_count, WalkParams walk, int with_walk, void *a_out, void *b_out) {
    extern __shared__ uint32_t s_limbs[];
    const uint32_t *limbs;
    if constexpr (kParam) {
        limbs = kl.limb;
    } else {
        const bool in_shared = nlimbs <= kMaxSharedLimbs;
        if (in_shared)
            for (int i = threadIdx.x; i < nlimbs; i += blockDim.x) s_limbs[i] = klimbs[i];
        __syncthreads();
        limbs = in_shared ? s_limbs : klimbs;
    }
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

// K'_g mod p for every group g of a chain (jobs of a batch sharing one L,
// their P ascending): K'_1 = P_1#/L, K'_g = K'_(g-1) * S_g with S_g the
// product of the primes in (P_(g-1), P_g] that do not divide L.  Per prime:
// Horner over each segment's limbs, most significant first (u <- REDC(u R^2
// + limb) leaves S_g R^-1; one more REDC with R^2 gives S_g), and the
// running product r_g = REDC(acc * S_g) with acc = r_(g-1) R (Montgomery
// form, one REDC with R^2).  One pass over K'_G's limbs serves every group,
// instead of one reduction of each K'_g.  Writes r_g at r_out[g * stride + i]
// and R^2 mod p at r2_out[i] (R = 2^32 or 2^64, the primes' width).
// The segments' limbs and then their G + 1 offsets arrive in the launch's
// parameters (kl) when they fit, else from seg_limbs / seg_off through
// shared memory.
template <bool kWide, bool kParam>
__global__ void __launch_bounds__(kKmodThreads)
    kmod_chain_kernel(const __grid_constant__ KLimbs<kParam ? kParamLimbs : 1> kl,
                      const uint32_t *__restrict__ seg_limbs, const uint32_t *__restrict__ seg_off, int G,
                      int nlimbs, uint64_t base, const uint32_t *__restrict__ off, uint64_t n, void *r_out,
                      void *r2_out) {
    extern __shared__ uint32_t s_words[];  // nlimbs limbs, then G + 1 segment offsets
    const uint32_t *s_limbs;
    if constexpr (kParam) {
        s_limbs = kl.limb;
    } else {
        for (int i = threadIdx.x; i < nlimbs; i += blockDim.x) s_words[i] = seg_limbs[i];
        for (int i = threadIdx.x; i <= G; i += blockDim.x) s_words[nlimbs + i] = seg_off[i];
        __syncthreads();
        s_limbs = s_words;
    }
    const uint32_t *so = s_limbs + nlimbs;
    if (!kWide) {
        uint32_t *ro = (uint32_t *)r_out;
        const uint64_t idx0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kChainPrimesPerThread;
        if (idx0 >= n) return;
        uint32_t p[kChainPrimesPerThread], pinv[kChainPrimesPerThread], r2[kChainPrimesPerThread],
            acc[kChainPrimesPerThread];
        bool lazy = true;
#pragma unroll
        for (int k = 0; k < kChainPrimesPerThread; k++) {
            p[k] = idx0 + k < n ? (uint32_t)(base + off[idx0 + k]) : 3u;  // pad with a prime
            pinv[k] = neg_inv32(p[k]);
            r2[k] = r2_from_r1(pow32_mod(p[k]), p[k], pinv[k]);
            acc[k] = 0;
            lazy = lazy && p[k] < 0x80000000u;
        }
        for (int g = 0; g < G; g++) {
            uint32_t u[kChainPrimesPerThread];
#pragma unroll
            for (int k = 0; k < kChainPrimesPerThread; k++) u[k] = 0;
            const int lo = (int)so[g], hi = (int)so[g + 1];
            if (lazy) {
                for (int i = hi - 1; i >= lo; i--) {
                    const uint32_t l = s_limbs[i];
#pragma unroll
                    for (int k = 0; k < kChainPrimesPerThread; k++)
                        u[k] = redc32_lazy((uint64_t)u[k] * r2[k] + l, p[k], pinv[k]);
                }
#pragma unroll
                for (int k = 0; k < kChainPrimesPerThread; k++)
                    if (u[k] >= p[k]) u[k] -= p[k];
            } else {
                for (int i = hi - 1; i >= lo; i--) {
                    const uint32_t l = s_limbs[i];
#pragma unroll
                    for (int k = 0; k < kChainPrimesPerThread; k++)
                        u[k] = redc32((uint64_t)u[k] * r2[k] + l, p[k], pinv[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < kChainPrimesPerThread; k++) {
                const uint32_t sg = redc32((uint64_t)u[k] * r2[k], p[k], pinv[k]);       // S_g mod p
                const uint32_t r = g ? redc32((uint64_t)acc[k] * sg, p[k], pinv[k]) : sg;  // K'_g mod p
                if (idx0 + k < n) ro[(uint64_t)g * n + idx0 + k] = r;
                acc[k] = redc32((uint64_t)r * r2[k], p[k], pinv[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < kChainPrimesPerThread; k++)
            if (idx0 + k < n) ((uint32_t *)r2_out)[idx0 + k] = r2[k];
    } else {
        uint64_t *ro = (uint64_t *)r_out;
        const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (idx >= n) return;
        const uint64_t p = base + off[idx];
        const uint64_t pinv = neg_inv64(p);
        uint64_t r1, r2;  // 2^64 and 2^128 mod p
        pow64_128_mod(p, r1, r2);
        uint64_t acc = 0;
        for (int g = 0; g < G; g++) {
            const int lo = (int)so[g], nl = (int)so[g + 1] - lo;
            uint64_t u = 0;
            for (int i = (nl + 1) / 2 - 1; i >= 0; i--) {
                uint64_t w = s_limbs[lo + 2 * i];
                if (2 * i + 1 < nl) w |= (uint64_t)s_limbs[lo + 2 * i + 1] << 32;
                const uint64_t lo2 = u * r2 + w;
                const uint64_t hi = umulhi64(u, r2) + (lo2 < w);
                u = redc64(hi, lo2, p, pinv);
            }
            const uint64_t sg = montmul64(u, r2, p, pinv);
            const uint64_t r = g ? montmul64(acc, sg, p, pinv) : sg;
            ro[(uint64_t)g * n + idx] = r;
            acc = montmul64(r, r2, p, pinv);
        }
        ((uint64_t *)r2_out)[idx] = r2;
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

// Least significant limb first once the cheaper step (an add, a multiply and
// a multiply-add, against a multiply-add, a multiply and a multiply-add)
// outweighs the R^(n+1) power.
bool kmod_lsb(int nlimbs, bool wide, int lsb_min_limbs) {
    const int lsb_min = lsb_min_limbs > 0 ? (wide ? std::max(1, lsb_min_limbs * 3 / 4) : lsb_min_limbs)
                                          : (wide ? kLsbMinLimbsWide : kLsbMinLimbs);
    return nlimbs >= lsb_min;
}

cudaError_t kmod_window(const uint32_t *d_klimbs, int nlimbs, uint64_t base, const uint32_t *d_off,
                        const unsigned long long *d_range, uint64_t max_count,
                        const WalkParams *walk, void *d_a, void *d_b, bool wide, cudaStream_t stream,
                        int lsb_min_limbs, const uint32_t *h_klimbs) {
    if (max_count == 0) return cudaSuccess;
    const WalkParams wp = walk ? *walk : WalkParams{};
    const int ww = walk != nullptr;
    const uint64_t per_thread = wide ? 1 : kPrimesPerThread;
    const uint64_t threads = (max_count + per_thread - 1) / per_thread;
    const unsigned blocks = (unsigned)((threads + kKmodThreads - 1) / kKmodThreads);
    const size_t smem = nlimbs <= kMaxSharedLimbs ? (size_t)nlimbs * sizeof(uint32_t) : 0;
    const bool lsb = kmod_lsb(nlimbs, wide, lsb_min_limbs);
    if (h_klimbs && nlimbs <= kParamLimbs) {
        KLimbs<kParamLimbs> kl;
        memcpy(kl.limb, h_klimbs, (size_t)nlimbs * sizeof(uint32_t));
        auto go = [&](auto kernel) {
            kernel<<<blocks, kKmodThreads, 0, stream>>>(kl, d_klimbs, nlimbs, base, d_off, d_range, max_count, wp,
                                                        ww, d_a, d_b);
        };
        if (wide && lsb) go(kmod_kernel<true, true, true>);
        else if (wide) go(kmod_kernel<true, false, true>);
        else if (lsb) go(kmod_kernel<false, true, true>);
        else go(kmod_kernel<false, false, true>);
        return cudaGetLastError();
    }
    const KLimbs<1> none{};
    auto go = [&](auto kernel) {
        kernel<<<blocks, kKmodThreads, smem, stream>>>(none, d_klimbs, nlimbs, base, d_off, d_range, max_count, wp,
                                                       ww, d_a, d_b);
    };
    if (wide && lsb) go(kmod_kernel<true, true, false>);
    else if (wide) go(kmod_kernel<true, false, false>);
    else if (lsb) go(kmod_kernel<false, true, false>);
    else go(kmod_kernel<false, false, false>);
    return cudaGetLastError();
}

cudaError_t kmod_list32(const uint32_t *d_klimbs, int nlimbs, const uint32_t *d_q, uint32_t n,
                        uint32_t *d_r, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    kmod_list_kernel<<<(n + kKmodThreads - 1) / kKmodThreads, kKmodThreads, 0, stream>>>(
        d_klimbs, nlimbs, d_q, n, d_r);
    return cudaGetLastError();
}

cudaError_t kmod_chain(const uint32_t *d_seg_limbs, const uint32_t *d_seg_off, int G, int nlimbs, uint64_t base,
                       const uint32_t *d_off, uint64_t n, void *d_r, void *d_r2, bool wide, cudaStream_t stream,
                       const uint32_t *h_seg_limbs, const uint32_t *h_seg_off) {
    if (n == 0 || G == 0) return cudaSuccess;
    const uint64_t per_thread = wide ? 1 : kChainPrimesPerThread;
    const uint64_t threads = (n + per_thread - 1) / per_thread;
    const unsigned blocks = (unsigned)((threads + kKmodThreads - 1) / kKmodThreads);
    if (nlimbs + G + 1 > kMaxSharedLimbs) return cudaErrorInvalidValue;
    if (h_seg_limbs && h_seg_off && nlimbs + G + 1 <= kParamLimbs) {
        KLimbs<kParamLimbs> kl;
        memcpy(kl.limb, h_seg_limbs, (size_t)nlimbs * sizeof(uint32_t));
        memcpy(kl.limb + nlimbs, h_seg_off, (size_t)(G + 1) * sizeof(uint32_t));
        if (wide)
            kmod_chain_kernel<true, true><<<blocks, kKmodThreads, 0, stream>>>(kl, d_seg_limbs, d_seg_off, G, nlimbs,
                                                                               base, d_off, n, d_r, d_r2);
        else
            kmod_chain_kernel<false, true><<<blocks, kKmodThreads, 0, stream>>>(kl, d_seg_limbs, d_seg_off, G, nlimbs,
                                                                                base, d_off, n, d_r, d_r2);
        return cudaGetLastError();
    }
    const size_t smem = (size_t)(nlimbs + G + 1) * sizeof(uint32_t);
    const KLimbs<1> none{};
    if (wide)
        kmod_chain_kernel<true, false><<<blocks, kKmodThreads, smem, stream>>>(none, d_seg_limbs, d_seg_off, G, nlimbs,
                                                                               base, d_off, n, d_r, d_r2);
    else
        kmod_chain_kernel<false, false><<<blocks, kKmodThreads, smem, stream>>>(none, d_seg_limbs, d_seg_off, G,
                                                                                nlimbs, base, d_off, n, d_r, d_r2);
    return cudaGetLastError();
}

}  // namespace pg
