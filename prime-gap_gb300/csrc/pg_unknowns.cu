// Unknowns as binary lists, for the next consumer (gap_stats) without a text
// parse on the host.
//
// gap_stats reads an unknowns file line by line and turns each line into two
// lists of distances with parse_unknown_line (gap_common.cpp:1186-1360, called
// from run_gap_file, gap_stats.cpp:1181-1290); for P=1511 with bitcompressed
// rows the reference notes that this parse is over half of its runtime
// (gap_stats.cpp:1254).  Here the lists come either straight from a sieved
// job's device lists (no text at all), or from a device parse of file bytes of
// any of the three formats.
//
// Output layout (one block, copied to the host in one transfer):
//   u64 m[rows] | u64 start[rows] | u32 n_prev[rows] | u32 n_next[rows] | u32 dist[total]
// row i: n_prev[i] distances of the -X unknowns, then n_next[i] of the +X
// unknowns, each side nearest first, at dist[start[i]...].
#include <string>

#include "pg_host.h"

namespace pg {
namespace {

constexpr uint64_t kChunk = 256;  // text bytes per thread when finding line ends

__global__ void count_lines_kernel(const char *__restrict__ text, uint64_t len, uint64_t *counts,
                                   uint64_t nchunks) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const uint64_t b = c * kChunk, e = min(b + kChunk, len);
    uint64_t n = 0;
    for (uint64_t i = b; i < e; i++) n += text[i] == '\n';
    counts[c] = n;
}

__global__ void line_ends_kernel(const char *__restrict__ text, uint64_t len, const uint64_t *offsets,
                                 uint64_t nchunks, uint64_t rows, uint64_t *line_end) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const uint64_t b = c * kChunk, e = min(b + kChunk, len);
    uint64_t k = offsets[c];
    for (uint64_t i = b; i < e; i++)
        if (text[i] == '\n') {
            if (k < rows) line_end[k] = i;
            k++;
        }
}

// istream-like reads inside one line [p, end)
struct Reader {
    const char *p, *end;
    __device__ void ws() {
        while (p < end && *p == ' ') p++;
    }
    // an integer with an optional sign; false if there is no digit
    __device__ bool num(int &sign, uint64_t &v) {
        ws();
        sign = 1;
        if (p < end && (*p == '-' || *p == '+')) {
            sign = *p == '-' ? -1 : 1;
            p++;
        }
        if (p >= end || *p < '0' || *p > '9') return false;
        v = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            v = v * 10 + (uint64_t)(*p - '0');
            p++;
        }
        return true;
    }
    // a token of n characters followed by a space
    __device__ bool tok(char c0, char c1, int n) {
        ws();
        if (end - p < n + 1) return false;
        if (p[0] != c0 || (n == 2 && p[1] != c1)) return false;
        p += n;
        return *p == ' ';
    }
};

struct ParseDev {
    const char *text;
    const uint64_t *line_end;  // rows
    uint64_t rows;
    int compression;
    uint32_t sl;
    uint32_t H;                // live offsets per side
    const uint32_t *dist_tab;  // their distances, ascending
    uint32_t nq;               // odd primes of d
    uint32_t q[16], kq[16];    // the primes and K mod each
    // per row
    uint64_t *m, *body, *total;
    uint32_t *n_prev, *n_next;
    unsigned long long *error;  // first bad row + 1 (0 = none)
};

__device__ void flag(const ParseDev &pd, uint64_t row) {
    atomicCAS(pd.error, 0ull, (unsigned long long)row + 1);
}

// Header of each line: m and the counts (gap_common.cpp:1199-1210, 1256-1266, 1290-1301).
__global__ void headers_kernel(ParseDev pd) {
    const uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= pd.rows) return;
    const uint64_t b = row ? pd.line_end[row - 1] + 1 : 0;
    Reader r;
    r.p = pd.text + b;
    r.end = pd.text + pd.line_end[row];
    int sg = 0, sa = 0, sc = 0;
    uint64_t m = 0, a = 0, c = 0;
    bool ok = r.num(sg, m) && sg > 0 && r.tok(':', 0, 1);
    if (pd.compression == 2) {
        ok = ok && r.num(sa, a) && sa > 0 && a > 0 && r.num(sc, c) && sc > 0 && r.tok('|', '|', 2);
        if (ok) ok = (uint64_t)(r.end - (r.p + 1)) == c;
        pd.n_prev[row] = 0;
        pd.n_next[row] = 0;
        pd.total[row] = ok ? a : 0;
    } else {
        ok = ok && r.num(sa, a) && sa < 0 && r.num(sc, c) && sc > 0 && r.tok('|', 0, 1);
        if (ok && pd.compression == 1) ok = (uint64_t)(r.end - (r.p + 1)) == 2 * a + 3 + 2 * c;
        pd.n_prev[row] = ok ? (uint32_t)a : 0;
        pd.n_next[row] = ok ? (uint32_t)c : 0;
        pd.total[row] = ok ? a + c : 0;
    }
    pd.m[row] = m;
    pd.body[row] = ok ? (uint64_t)(r.p + 1 - pd.text) : 0;  // after the space that follows '|' or "||"
    if (!ok) flag(pd, row);
}

__device__ __forceinline__ bool is_digit(char c) { return c >= '0' && c <= '9'; }

// One warp per line.
__global__ void bodies_kernel(ParseDev pd, const uint64_t *__restrict__ start, uint32_t *__restrict__ dist) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= pd.rows) return;
    const uint64_t b = pd.body[row], e = pd.line_end[row];
    if (b == 0) return;  // the header failed (flagged)
    const uint32_t lt = (1u << lane) - 1;
    const char *text = pd.text;
    uint32_t *out = dist + start[row];

    if (pd.compression == 0) {
        // " -x ... | +y ...": a sign preceded by a space starts a token
        const uint32_t np = pd.n_prev[row], nn = pd.n_next[row];
        uint32_t k0 = 0, k1 = 0;
        for (uint64_t i0 = b; i0 < e; i0 += 32) {
            const uint64_t i = i0 + lane;
            const char c = i < e ? text[i] : 0;
            const bool sign = c == '-' || c == '+';
            const bool start_tok = sign && text[i - 1] == ' ';  // i >= b >= 1
            const uint32_t m0 = __ballot_sync(0xffffffffu, start_tok && c == '-');
            const uint32_t m1 = __ballot_sync(0xffffffffu, start_tok && c == '+');
            if (start_tok) {
                uint32_t v = 0;
                uint64_t j = i + 1;
                while (j < e && is_digit(text[j])) {
                    v = v * 10 + (uint32_t)(text[j] - '0');
                    j++;
                }
                if (c == '-') {
                    const uint32_t k = k0 + __popc(m0 & lt);
                    if (k < np) out[k] = v;
                } else {
                    const uint32_t k = k1 + __popc(m1 & lt);
                    if (k < nn) out[np + k] = v;
                }
            }
            k0 += __popc(m0);
            k1 += __popc(m1);
        }
        if (lane == 0 && (k0 != np || k1 != nn)) flag(pd, row);
        return;
    }

    if (pd.compression == 1) {
        // "| " 2a bytes " | " 2b bytes: each pair a delta, the distances
        // their running sums (combined_sieve.cpp:1396-1417)
        const uint32_t np = pd.n_prev[row], nn = pd.n_next[row];
        if (lane == 0 && (text[b + 2ull * np] != ' ' || text[b + 2ull * np + 1] != '|' ||
                          text[b + 2ull * np + 2] != ' '))
            flag(pd, row);
        for (int side = 0; side < 2; side++) {
            const uint32_t n = side ? nn : np;
            const uint64_t base = side ? b + 2ull * np + 3 : b;
            uint32_t carry = 0;
            for (uint32_t k0 = 0; k0 < n; k0 += 32) {
                const uint32_t k = k0 + lane;
                uint32_t v = 0;
                if (k < n) {
                    const uint32_t hi = (unsigned char)text[base + 2ull * k];
                    const uint32_t lo = (unsigned char)text[base + 2ull * k + 1];
                    v = (hi - 48) * 128 + (lo - 48);
                }
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
                    if (lane >= (uint32_t)o) v += t;
                }
                if (k < n) out[(side ? np : 0) + k] = carry + v;
                carry += __shfl_sync(0xffffffffu, v, 31);
            }
        }
        return;
    }

    // compression 2 (gap_common.cpp:1212-1288): over the live offsets in
    // increasing x that are not multiples of an odd prime of d for this m,
    // one flag bit each, 7 per byte; a clear bit is an unknown.  The low
    // side runs x = SL - dist (farthest first), then the high side x = SL + dist.
    const uint64_t m = pd.m[row];
    uint32_t first[16];
    for (uint32_t t = 0; t < pd.nq; t++) {
        // m*K + (x - SL) = 0 (mod q)  <=>  x = SL - m*K (mod q)
        const uint32_t q = pd.q[t];
        const uint32_t mk = (uint32_t)((m % q) * pd.kq[t] % q);
        first[t] = (pd.sl % q + q - mk) % q;
    }
    const unsigned char *raw = (const unsigned char *)text + b;
    const uint32_t H = pd.H, sl = pd.sl;
    const uint64_t nbytes = e - b;
    // pass 0 counts the low side's unknowns (np), pass 1 writes them nearest
    // first (out[np - 1 - j]), pass 2 writes the high side after them; the
    // flag index runs on from the low side into the high side
    uint32_t np = 0, bit_idx = 0, found = 0;
    for (int pass = 0; pass < 3; pass++) {
        const int side = pass == 2;
        if (pass < 2) bit_idx = 0;
        found = 0;
        for (uint32_t h0 = 0; h0 < H; h0 += 32) {
            const uint32_t k = h0 + lane;
            bool fc = false;
            uint32_t x = 0;
            if (k < H) {
                const uint32_t d = pd.dist_tab[side ? k : H - 1 - k];
                x = side ? sl + d : sl - d;
                fc = true;
                for (uint32_t t = 0; t < pd.nq; t++) fc = fc && (x % pd.q[t]) != first[t];
            }
            const uint32_t fm = __ballot_sync(0xffffffffu, fc);
            bool unknown = false;
            if (fc) {
                const uint32_t idx = bit_idx + __popc(fm & lt);
                const uint64_t byte = idx / 7;
                unknown = byte < nbytes && ((raw[byte] >> (idx % 7)) & 1u) == 0;
            }
            const uint32_t um = __ballot_sync(0xffffffffu, unknown);
            if (unknown && pass > 0) {
                const uint32_t j = found + __popc(um & lt);
                if (side == 0) out[np - 1 - j] = sl - x;
                else out[np + j] = x - sl;
            }
            bit_idx += __popc(fm);
            found += __popc(um);
        }
        if (pass == 0) np = found;
    }
    if (lane == 0) {
        pd.n_prev[row] = np;
        pd.n_next[row] = found;
        if ((uint64_t)np + found != pd.total[row] || (uint64_t)(bit_idx + 6) / 7 != nbytes) flag(pd, row);
    }
}

// Device lists of a sieved job (compression 0/1) into the packed layout.
__global__ void gather_kernel(const uint32_t *__restrict__ lists, const uint32_t *__restrict__ counts,
                              uint32_t H, uint64_t rows, const uint64_t *__restrict__ start,
                              uint32_t *__restrict__ dist) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= rows) return;
    const uint32_t np = counts[2 * row], nn = counts[2 * row + 1];
    const uint32_t *src = lists + row * 2ull * H;
    uint32_t *dst = dist + start[row];
    for (uint32_t k = lane; k < np; k += 32) dst[k] = src[k];
    for (uint32_t k = lane; k < nn; k += 32) dst[np + k] = src[H + k];
}

__global__ void totals_kernel(const uint32_t *__restrict__ counts, uint64_t rows, uint64_t *total,
                              uint32_t *n_prev, uint32_t *n_next) {
    const uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    const uint32_t a = counts[2 * row], b = counts[2 * row + 1];
    n_prev[row] = a;
    n_next[row] = b;
    total[row] = (uint64_t)a + b;
}

__global__ void m_kernel(const uint32_t *__restrict__ valid_mi, uint64_t rows, uint64_t mstart, uint64_t *m) {
    const uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row < rows) m[row] = mstart + valid_mi[row];
}

unsigned grid(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace pg

using namespace pgh;

namespace {


// Copy the packed block to library-owned pinned memory and fill *out.
int packed_fetch(pgs_ctx *ctx, const PackedLists &pk, uint64_t total, cudaStream_t s, pgs_unknowns *out) {
    const uint64_t rows = pk.rows;
    const size_t bytes = rows * 24 + total * 4;
    size_t cap = 0;
    char *host = pinned_pool().get(bytes + 64, &cap);
    if (!host) {
        ctx->err = "cudaMallocHost failed";
        return PGS_ENOMEM;
    }
    cudaError_t e = cudaMemcpyAsync(host, pk.block.p, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        pinned_pool().put(host, cap);
        return fail(ctx, e, "unknowns copy");
    }
    out->rows = rows;
    out->m = (uint64_t *)host;
    out->start = (uint64_t *)(host + rows * 8);
    out->n_prev = (uint32_t *)(host + rows * 16);
    out->n_next = (uint32_t *)(host + rows * 20);
    out->dist = (uint32_t *)(host + rows * 24);
    out->total = total;
    out->internal = new PinnedOwner{cap};
    return PGS_OK;
}

// Parse text already on the device (d_text, len bytes) for the derived job h
// into the packed block pk (pk.total set).
int parse_device_text_packed(pgs_ctx *ctx, const HostJob &h, const char *d_text, uint64_t len, cudaStream_t s,
                             PackedLists &pk) {
    const uint64_t rows = h.valid_mi.size();
    const uint64_t nchunks = (len + pg::kChunk - 1) / pg::kChunk;
    DevBuf counts, offs, tmp, line_end, body, tot, err, misc, dist_tab;
    DevBuf *bufs[] = {&counts, &offs, &tmp, &line_end, &body, &tot, &err, &misc, &dist_tab};
    for (DevBuf *b : bufs) b->pool = &ctx->dpool;
    pk.block.pool = &ctx->dpool;
    auto cleanup = [&] {
        cudaStreamSynchronize(s);
        for (DevBuf *b : bufs) b->release();
    };
    // no line holds more unknowns than its job's 2H live offsets, nor more
    // than one per two bytes (plain and RLE) or seven per byte (bitcompressed)
    const uint64_t max_total = std::min<uint64_t>(8 * len + 8, rows * 2ull * h.H + 1);
    cudaError_t e = counts.ensure(nchunks * 8 + 8);
    if (e == cudaSuccess) e = offs.ensure(nchunks * 8 + 8);
    if (e == cudaSuccess) e = tmp.ensure(pg::scan_tmp_words(std::max<uint64_t>(nchunks, rows)) * 8 + 8);
    if (e == cudaSuccess) e = line_end.ensure(rows * 8 + 8);
    if (e == cudaSuccess) e = body.ensure(rows * 8 + 8);
    if (e == cudaSuccess) e = tot.ensure(rows * 8 + 8);
    if (e == cudaSuccess) e = err.ensure(16);
    if (e == cudaSuccess) e = misc.ensure(16);
    if (e == cudaSuccess) e = packed_alloc(pk, rows, max_total);
    if (e == cudaSuccess) e = upload(dist_tab, h.dist, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(err.p, 0, 16, s);
    if (e != cudaSuccess) {
        cleanup();
        return fail(ctx, e, "parse buffers");
    }
    // line ends: per-chunk newline counts, their prefix sum, then positions
    uint64_t lines = 0;
    if (nchunks) {
        pg::count_lines_kernel<<<pg::grid(nchunks, 256), 256, 0, s>>>(d_text, len, counts.as<uint64_t>(),
                                                                     nchunks);
        e = pg::scan_u64(counts.as<uint64_t>(), offs.as<uint64_t>(), misc.as<uint64_t>(), nchunks,
                         tmp.as<uint64_t>(), s);
        if (e == cudaSuccess) {
            pg::line_ends_kernel<<<pg::grid(nchunks, 256), 256, 0, s>>>(d_text, len, offs.as<uint64_t>(), nchunks,
                                                                       rows, line_end.as<uint64_t>());
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(&lines, misc.p, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess) {
        cleanup();
        return fail(ctx, e, "parse line ends");
    }
    if (lines != rows) {
        cleanup();
        ctx->err = "unknowns text has " + std::to_string(lines) + " lines, the job has " +
                   std::to_string(rows) + " valid m";
        return PGS_EINVAL;
    }
    pg::ParseDev pd{};
    pd.text = d_text;
    pd.line_end = line_end.as<uint64_t>();
    pd.rows = rows;
    pd.compression = h.job.compression;
    pd.sl = h.job.sieve_length;
    pd.H = h.H;
    pd.dist_tab = dist_tab.as<uint32_t>();
    pd.nq = (uint32_t)std::min<size_t>(h.dq.size(), 16);
    for (uint32_t t = 0; t < pd.nq; t++) {
        pd.q[t] = h.dq[t];
        uint64_t r = 0;  // K mod q from the limbs, most significant first
        for (size_t i = h.klimbs.size(); i-- > 0;) r = ((r << 32) | h.klimbs[i]) % h.dq[t];
        pd.kq[t] = (uint32_t)r;
    }
    pd.m = pk.m;
    pd.body = body.as<uint64_t>();
    pd.total = tot.as<uint64_t>();
    pd.n_prev = pk.n_prev;
    pd.n_next = pk.n_next;
    pd.error = err.as<unsigned long long>();
    uint64_t total = 0, bad = 0;
    if (rows) {
        pg::headers_kernel<<<pg::grid(rows, 256), 256, 0, s>>>(pd);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = pg::scan_u64(pd.total, pk.start, misc.as<uint64_t>(), rows, tmp.as<uint64_t>(), s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, misc.p, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, err.p, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess && !bad && total > max_total) {
            cleanup();
            ctx->err = "unknowns text claims " + std::to_string(total) + " unknowns, more than the " +
                       std::to_string(max_total) + " its job can have";
            return PGS_EINVAL;
        }
        if (e == cudaSuccess && !bad) {
            pg::bodies_kernel<<<pg::grid(rows * 32, 256), 256, 0, s>>>(pd, pk.start, pk.dist);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, err.p, 8, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    if (e != cudaSuccess) {
        cleanup();
        return fail(ctx, e, "parse unknowns");
    }
    if (bad) {
        cleanup();
        ctx->err = "malformed unknowns line " + std::to_string(bad - 1);
        return PGS_EINVAL;
    }
    pk.total = total;
    cleanup();
    return PGS_OK;
}

int parse_device_text(pgs_ctx *ctx, const HostJob &h, const char *d_text, uint64_t len, cudaStream_t s,
                      pgs_unknowns *out) {
    PackedLists pk;
    int rc = parse_device_text_packed(ctx, h, d_text, len, s, pk);
    if (rc == PGS_OK) rc = packed_fetch(ctx, pk, pk.total, s, out);
    cudaStreamSynchronize(s);
    pk.block.release();
    return rc;
}

}  // namespace

namespace pgh {

cudaError_t packed_alloc(PackedLists &pk, uint64_t rows, uint64_t max_total) {
    pk.rows = rows;
    cudaError_t e = pk.block.ensure(rows * 24 + max_total * 4 + 64);
    if (e) return e;
    char *b = pk.block.as<char>();
    pk.m = (uint64_t *)b;
    pk.start = (uint64_t *)(b + rows * 8);
    pk.n_prev = (uint32_t *)(b + rows * 16);
    pk.n_next = (uint32_t *)(b + rows * 20);
    pk.dist = (uint32_t *)(b + rows * 24);
    return cudaSuccess;
}

// A sieved job's lists as a packed device block (no host copy): the device
// lists of a plain or RLE job gathered in row order, or a bitcompressed job's
// device text decoded in place.  pk.total = entries of pk.dist.
int job_lists_device(pgs_ctx *ctx, pgs_prepared *pr, cudaStream_t s, PackedLists &pk) {
    const HostJob &h = pr->hj;
    pk.block.pool = &ctx->dpool;
    if (h.job.compression == 2) {
        uint64_t len = 0;
        CK(cudaMemcpyAsync(&len, pr->misc.p, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        return parse_device_text_packed(ctx, h, pr->text.as<char>(), len, s, pk);
    }
    const uint64_t rows = h.valid_mi.size();
    DevBuf tot, tmp, misc;
    DevBuf *bufs[] = {&tot, &tmp, &misc};
    for (DevBuf *b : bufs) b->pool = &ctx->dpool;
    auto cleanup = [&] {
        cudaStreamSynchronize(s);
        for (DevBuf *b : bufs) b->release();
    };
    cudaError_t e = packed_alloc(pk, rows, rows * 2ull * h.H);
    if (e == cudaSuccess) e = tot.ensure(rows * 8 + 8);
    if (e == cudaSuccess) e = tmp.ensure(pg::scan_tmp_words(rows) * 8 + 8);
    if (e == cudaSuccess) e = misc.ensure(16);
    uint64_t total = 0;
    if (e == cudaSuccess && rows) {
        const uint32_t *counts = pr->counts.as<uint32_t>();
        pg::totals_kernel<<<pg::grid(rows, 256), 256, 0, s>>>(counts, rows, tot.as<uint64_t>(), pk.n_prev,
                                                              pk.n_next);
        pg::m_kernel<<<pg::grid(rows, 256), 256, 0, s>>>(pr->valid_mi.as<uint32_t>(), rows, h.job.mstart, pk.m);
        e = pg::scan_u64(tot.as<uint64_t>(), pk.start, misc.as<uint64_t>(), rows, tmp.as<uint64_t>(), s);
        if (e == cudaSuccess)
            pg::gather_kernel<<<pg::grid(rows * 32, 256), 256, 0, s>>>(pr->lists.as<uint32_t>(), counts, h.H,
                                                                       rows, pk.start, pk.dist);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, misc.p, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cleanup();
    if (e != cudaSuccess) return fail(ctx, e, "job lists");
    pk.total = total;
    return PGS_OK;
}

}  // namespace pgh

extern "C" {

int pgs_parse_unknowns(pgs_ctx *ctx, const pgs_job *job, const char *text, uint64_t len,
                       pgs_unknowns *out) {
    if (!ctx || !job || !out || (!text && len)) return PGS_EINVAL;
    memset(out, 0, sizeof(*out));
    std::lock_guard<std::mutex> g(ctx->mu);
    HostJob h;
    int rc = derive(*job, h, ctx->err, true);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    const cudaStream_t s = ctx->stream;
    DevBuf d_text;
    d_text.pool = &ctx->dpool;
    CK(d_text.ensure(len + 1));
    if (len) {
        cudaError_t e = cudaMemcpyAsync(d_text.p, text, len, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            d_text.release();
            return fail(ctx, e, "unknowns upload");
        }
    }
    rc = parse_device_text(ctx, h, d_text.as<char>(), len, s, out);
    cudaStreamSynchronize(s);
    d_text.release();
    return rc;
}

int pgs_fetch_unknowns(pgs_ctx *ctx, pgs_prepared *pr, pgs_unknowns *out) {
    if (!ctx || !pr || !out || pr->ctx != ctx || !pr->ran) return PGS_EINVAL;
    memset(out, 0, sizeof(*out));
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    const cudaStream_t s = ctx->stream;
    PackedLists pk;
    int rc = job_lists_device(ctx, pr, s, pk);
    if (rc == PGS_OK) rc = packed_fetch(ctx, pk, pk.total, s, out);
    cudaStreamSynchronize(s);
    pk.block.release();
    return rc;
}

void pgs_unknowns_free(pgs_unknowns *u) {
    if (!u) return;
    if (u->m && u->internal) {
        auto *own = (PinnedOwner *)u->internal;
        pinned_pool().put((char *)u->m, own->cap);
        delete own;
    }
    memset(u, 0, sizeof(*u));
}

}  // extern "C"
