// pgs_large_hits_static: pgs_large_hits without any allocation.
//
// pgs_large_hits allocates (and frees) three device buffers per call: the
// hit lists and the hit counter.  Here they live in one file-scope __device__
// array of fixed size, so a call makes no cudaMalloc/cudaFree and no
// allocating library call.  Its address comes from cudaGetSymbolAddress,
// looked up once per device (with that device current) on the first call and
// cached; that first lookup may load the module, so the first call on a
// device belongs before any stream capture on it.  A cudaDeviceReset
// invalidates the cached address (as it does every context's streams and
// buffers): the library does not support a reset while it is in use.
//
// Limit: at most kStaticHitsMax hits are returned per call (cap above it is
// rejected with PGS_EINVAL).  The buffer is shared by every context on the
// device: calls that overlap in time (other threads or contexts on the same
// device) race on it and must be serialised by the caller; calls on one
// context are serialised by the context's lock.
#include <mutex>

#include "pg_host.h"

using namespace pgh;

namespace {

constexpr size_t kStaticHitsMax = 1u << 16;  // hits one call can return
constexpr size_t kCounterBytes = 256;        // hit counter, padded to keep the lists aligned
constexpr size_t kStaticBytes = kCounterBytes + kStaticHitsMax * sizeof(uint64_t) +
                                kStaticHitsMax * sizeof(uint32_t);  // 786,688 bytes

// layout: [counter (u64) | residues (u64 x kStaticHitsMax) | m indexes (u32 x kStaticHitsMax)]
static __device__ __align__(256) unsigned char g_hits_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
unsigned char *g_addr[kMaxDevices];

// Address of this device's buffer (the device must be current).
int scratch_address(pgs_ctx *ctx, unsigned char **out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices) {
        ctx->err = "device index out of range for the static hit buffer";
        return PGS_EINVAL;
    }
    std::lock_guard<std::mutex> g(g_addr_mu);
    if (!g_addr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_hits_scratch);
        if (e != cudaSuccess) return fail(ctx, e, "cudaGetSymbolAddress(g_hits_scratch)");
        g_addr[ctx->device] = (unsigned char *)p;
    }
    *out = g_addr[ctx->device];
    return PGS_OK;
}

}  // namespace

extern "C" int pgs_large_hits_static(pgs_ctx *ctx, uint64_t M, uint32_t max_mi, uint32_t SL,
                                     uint64_t prime, uint64_t base_r, uint32_t *mi_out,
                                     uint64_t *mod_out, size_t cap, size_t *count) {
    if (!ctx || !count) return PGS_EINVAL;
    if (prime <= 4ull * SL + 2 || prime >= (1ull << 46) || base_r == 0 || base_r >= prime)
        return PGS_EINVAL;
    if (cap > kStaticHitsMax) {
        ctx->err = "cap exceeds the static hit buffer (65536 hits)";
        return PGS_EINVAL;
    }
    if (cap && (!mi_out || !mod_out)) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    unsigned char *base = nullptr;
    int rc = scratch_address(ctx, &base);
    if (rc != PGS_OK) return rc;
    auto *cnt = (unsigned long long *)base;
    auto *mods = (uint64_t *)(base + kCounterBytes);
    auto *mis = (uint32_t *)(base + kCounterBytes + kStaticHitsMax * sizeof(uint64_t));
    cudaStream_t s = ctx->stream;
    // the counter must start at zero (the kernel overwrites it, but a stale
    // value must never be read back if the launch fails)
    CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
    CK(pg::tools_large_hits(M, max_mi, SL, prime, base_r, mis, mods, cap, cnt, s));
    uint64_t n = 0;
    CK(cudaMemcpyAsync(&n, cnt, sizeof n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const size_t w = n < cap ? (size_t)n : cap;
    if (w) {
        CK(cudaMemcpyAsync(mi_out, mis, w * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(mod_out, mods, w * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    *count = n;
    return PGS_OK;
}
