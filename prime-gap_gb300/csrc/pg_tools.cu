// Device batches of the reference's number-theory primitives, exposed through
// the C ABI for callers that need them one by one (and for parity tests):
// K mod q over an explicit prime list, the Euclid modulo search, and the hit
// enumeration of one prime.
#include "pg_arith.cuh"
#include "pg_internal.h"

namespace pg {

namespace {

__global__ void kmod_list64_kernel(const uint32_t *__restrict__ limbs, int n, const uint64_t *q,
                                   size_t count, uint64_t *out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t p = q[i];
    if (p < 0x80000000ull) {
        uint32_t pinv, r2;
        out[i] = kmod32(limbs, n, (uint32_t)p, pinv, r2);
    } else {
        out[i] = kmod64(limbs, n, p);
    }
}

__global__ void modsearch_kernel(const uint64_t *p, const uint64_t *a, const uint64_t *l,
                                 const uint64_t *r, uint64_t *k, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    k[i] = modsearch64(p[i], a[i], l[i], r[i]).k;
}

struct Collect {
    uint32_t *mi_out;
    uint64_t *mod_out;
    size_t cap;
    size_t n;
    __device__ void operator()(uint64_t mi, uint64_t y) {
        if (n < cap) {
            mi_out[n] = (uint32_t)mi;
            mod_out[n] = y;
        }
        n++;
    }
};

__global__ void large_hits_kernel(uint64_t M, uint32_t max_mi, uint32_t sl, uint64_t p,
                                  uint64_t r, uint32_t *mi_out, uint64_t *mod_out, size_t cap,
                                  unsigned long long *count) {
    Collect c{mi_out, mod_out, cap, 0};
    const uint64_t two_sl = 2ull * sl;
    if (p < 0xFFFFFFFFull) {
        uint32_t p32 = (uint32_t)p, r32 = (uint32_t)r;
        // y(0) = (r*M + SL) mod p
        uint32_t y = (uint32_t)((((M % p32) * (uint64_t)r32) % p32 + sl) % p32);
        enumerate_hits_cf<uint32_t>(p32, r32, y, 0, max_mi, (uint32_t)two_sl, c);
    } else {
        uint64_t y = mulmod_u64(M % p, r, p, 1.0 / (double)p) + sl;
        if (y >= p) y -= p;
        enumerate_hits_cf<uint64_t>(p, r, y, 0, max_mi, two_sl, c);
    }
    *count = c.n;
}

// Independent IMAD chains: 8 per thread, 16-way unrolled.
__global__ void __launch_bounds__(256) imad_peak_kernel(uint32_t a, uint32_t b, int iters,
                                                        uint32_t *sink) {
    uint32_t x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    uint32_t x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = x0 * a + b;
            x1 = x1 * a + b;
            x2 = x2 * a + b;
            x3 = x3 * a + b;
            x4 = x4 * a + b;
            x5 = x5 * a + b;
            x6 = x6 * a + b;
            x7 = x7 * a + b;
        }
    }
    uint32_t v = x0 ^ x1 ^ x2 ^ x3 ^ x4 ^ x5 ^ x6 ^ x7;
    if (v == 0x9E3779B9u) sink[blockIdx.x] = v;
}

}  // namespace

cudaError_t tools_imad_peak(double *imad_per_s, cudaStream_t stream) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint32_t *sink = nullptr;
    cudaError_t e = cudaMalloc(&sink, 65536 * sizeof(uint32_t));
    if (e) return e;
    const int blocks = sms * 8, threads = 256, iters = 4096;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    imad_peak_kernel<<<blocks, threads, 0, stream>>>(0x9E3779B1u, 12345u, 64, sink);  // warm-up
    double best = 0;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(t0, stream);
        imad_peak_kernel<<<blocks, threads, 0, stream>>>(0x9E3779B1u, 12345u, iters, sink);
        cudaEventRecord(t1, stream);
        e = cudaEventSynchronize(t1);
        if (e) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, t0, t1);
        double ops = (double)blocks * threads * iters * 16.0 * 8.0;
        double rate = ops / (ms * 1e-3);
        if (rate > best) best = rate;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(sink);
    *imad_per_s = best;
    return e ? e : cudaGetLastError();
}

cudaError_t tools_kmod_list64(const uint32_t *d_limbs, int n, const uint64_t *d_q, size_t count,
                              uint64_t *d_out, cudaStream_t stream) {
    if (!count) return cudaSuccess;
    kmod_list64_kernel<<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(d_limbs, n, d_q, count,
                                                                           d_out);
    return cudaGetLastError();
}

cudaError_t tools_modsearch(const uint64_t *p, const uint64_t *a, const uint64_t *l,
                            const uint64_t *r, uint64_t *k, size_t n, cudaStream_t stream) {
    if (!n) return cudaSuccess;
    modsearch_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(p, a, l, r, k, n);
    return cudaGetLastError();
}

cudaError_t tools_large_hits(uint64_t M, uint32_t max_mi, uint32_t sl, uint64_t p, uint64_t r,
                             uint32_t *mi_out, uint64_t *mod_out, size_t cap,
                             unsigned long long *count, cudaStream_t stream) {
    large_hits_kernel<<<1, 1, 0, stream>>>(M, max_mi, sl, p, r, mi_out, mod_out, cap, count);
    return cudaGetLastError();
}

}  // namespace pg
