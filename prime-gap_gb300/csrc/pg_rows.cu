// Row phase: small primes per m, merge with the large-prime marks, compaction
// of each m's unknown offsets, and the unknowns-file text.
//
// Small primes replace method2_small_primes (combined_sieve.cpp:1450-1603):
// for every m the multiples of each prime p <= 4*SL+2 (p > P, or p | d) are
// struck from the offsets of m*K + X.  A CTA holds the bitmaps of up to 32
// consecutive valid m in shared memory, over the offsets of the one parity
// that can be prime (m*K + X odd).  Odd primes dividing d stamp a per-word
// pattern that also initialises the bitmap; the other small primes are
// marked by one thread each, walking the CTA's m values with the residue
// update x0 <- x0 - r (mod p).
//
// The same CTA then ORs each row's large-prime bits (written by pg_large.cu,
// one per live offset in distance order) into the row's bitmap and compacts
// the live offsets left unmarked, nearest first on each side, into a per-row
// list; that replaces the coprime_prev/coprime_next walk of
// save_unknowns_method2 (combined_sieve.cpp:1289-1300, 1387-1438).
// format_rows then writes the rows' text in parallel at offsets given by a
// prefix sum of the per-row byte counts.
#include "pg_internal.h"

#include <algorithm>

namespace pg {

namespace {

constexpr int kRowThreads = 512;
constexpr int kMaxDPrimes = 16;

__device__ __forceinline__ uint32_t ndigits(uint64_t v) {
    uint32_t n = 1;
    while (v >= 10) {
        v /= 10;
        n++;
    }
    return n;
}

__device__ __forceinline__ uint32_t word_pattern(uint32_t q) {
    uint32_t m = 0;
    for (uint32_t b = 0; b < 32; b += q) m |= 1u << b;
    return m;
}

__global__ void __launch_bounds__(kRowThreads) rows_kernel(RowsDev rd, uint32_t rows_per_block,
                                                            uint32_t block0) {
    extern __shared__ uint32_t sh[];
    const JobDev &job = rd.job;
    const uint32_t nbw = (rd.nb + 31) / 32;
    const uint32_t r0 = (blockIdx.x + block0) * rows_per_block;
    if (r0 >= job.rows) return;
    const uint32_t nrows = min(rows_per_block, job.rows - r0);
    uint32_t *s_mi = sh + (size_t)rows_per_block * nbw;  // rows_per_block entries
    uint32_t *s_h0 = s_mi + rows_per_block;               // rows_per_block * kMaxDPrimes
    // bitcompressed rows also need the d-prime pattern alone
    uint32_t *s_pat = s_h0 + (size_t)rows_per_block * kMaxDPrimes;
    const uint32_t sl = job.sl, x_par = rd.x_par;

    for (uint32_t j = threadIdx.x; j < nrows; j += blockDim.x) s_mi[j] = rd.valid_mi[r0 + j];
    __syncthreads();

    // 1. patterns of the odd primes dividing d: start index per (row, q)
    for (uint32_t idx = threadIdx.x; idx < nrows * rd.nd; idx += blockDim.x) {
        uint32_t j = idx / rd.nd, t = idx % rd.nd;
        uint32_t q = rd.dq[t], rq = rd.dr[t];
        uint64_t m = job.mstart + s_mi[j];
        uint32_t mr = (uint32_t)(((m % q) * rq) % q);
        uint32_t x0 = (sl % q + q - mr) % q;  // p | m*K - SL + x
        if ((x0 & 1) != x_par) x0 += q;
        s_h0[j * kMaxDPrimes + t] = ((x0 - x_par) >> 1) % q;
    }
    __syncthreads();
    // Word w of row j has q's bits at b = (h0 - 32 w) mod q + k q (h0: the
    // row's first multiple): one thread per word for all the CTA's rows, so
    // 32 w mod q and q's word pattern are found once per (word, q) and each
    // row costs a subtraction.
    for (uint32_t w = threadIdx.x; w < nbw; w += blockDim.x) {
        for (uint32_t j = 0; j < nrows; j++) sh[j * nbw + w] = 0;
        for (uint32_t t = 0; t < rd.nd; t++) {
            const uint32_t q = rd.dq[t];
            const uint32_t pat = word_pattern(q), c = (32u * w) % q;
            for (uint32_t j = 0; j < nrows; j++) {
                const uint32_t h0 = s_h0[j * kMaxDPrimes + t];  // < q
                const uint32_t o = h0 >= c ? h0 - c : h0 + (q - c);
                if (o < 32) sh[j * nbw + w] |= pat << o;
            }
        }
        if (rd.compression == 2)
            for (uint32_t j = 0; j < nrows; j++) s_pat[j * nbw + w] = sh[j * nbw + w];
    }
    __syncthreads();

    // 2. other small primes, one thread per prime walking the CTA's m values
    const uint64_t sp_begin = rd.sp_range[0];
    const uint64_t ns = min((uint64_t)(rd.sp_range[1] - sp_begin), rd.sp_cap);
    const uint32_t mi_first = s_mi[0];
    for (uint64_t i = threadIdx.x; i < ns; i += blockDim.x) {
        const uint32_t p = rd.sp_base + rd.sp[sp_begin + i], r = rd.sr[i];
        const uint64_t m = job.mstart + mi_first;
        // (sl - m r) mod p, with 32-bit remainders where the operands fit
        const uint32_t mm = (m >> 32) ? (uint32_t)(m % p) : (uint32_t)m % p;
        const uint64_t prod = (uint64_t)mm * r;
        const uint32_t mr = (prod >> 32) ? (uint32_t)(prod % p) : (uint32_t)prod % p;
        const uint32_t sr = sl % p;
        uint32_t x0 = sr >= mr ? sr - mr : sr + (p - mr);
        // row by row (the same row across the warp): step the residue over
        // the m values since the previous row, then strike this row; with d
        // even every valid m is odd, so the step is 2r mod p per two m
        const uint32_t stride = job.walk.stride;
        const uint32_t rs = stride == 2 ? (r >= p - r ? r - (p - r) : r + r) : r;
        uint32_t mi_at = mi_first;
        for (uint32_t j = 0; j < nrows; j++) {
            const uint32_t mi = s_mi[j];
            for (; mi_at < mi; mi_at += stride) x0 = x0 >= rs ? x0 - rs : x0 + (p - rs);
            const uint32_t xs = x0 + (((x0 ^ x_par) & 1) ? p : 0);
            for (uint32_t h = (xs - x_par) >> 1; h < rd.nb; h += p)
                atomicOr(&sh[j * nbw + (h >> 5)], 1u << (h & 31));
        }
    }
    __syncthreads();

    // 3. merge with the large-prime bits and compact, one warp per row
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const uint32_t H = job.half_cols;
    if (rd.compression == 2) {
        // Bitcompressed rows (combined_sieve.cpp:1327-1385): over the offsets
        // in increasing X that are coprime to K and to every prime of d
        // (live and not in the d-prime pattern), the composite flags, 7 per
        // byte with bit 7 set.  The byte list goes to the row's list slot.
        for (uint32_t j = warp; j < nrows; j += nwarps) {
            const uint32_t row = r0 + j;
            const uint32_t *grow = job.comp + (uint64_t)row * job.pitch;
            uint8_t *bytes = (uint8_t *)(rd.lists + (uint64_t)row * 2 * H);
            uint32_t unk = 0, nbytes = 0, bit = 0, b = 0x80;
            for (uint32_t side = 0; side < 2; side++) {
                for (uint32_t h0 = 0; h0 < H; h0 += 32) {
                    // side 0 walks its columns backwards: increasing X
                    const uint32_t k = h0 + lane;
                    bool fc = false, composite = false;
                    if (k < H) {
                        const uint32_t h = side ? k : H - 1 - k;
                        const uint32_t d = rd.dist[h];
                        const uint32_t x = side ? sl + d : sl - d;
                        const uint32_t hx = (x - x_par) >> 1;
                        const uint32_t pat = (s_pat[j * nbw + (hx >> 5)] >> (hx & 31)) & 1;
                        const uint32_t sb = (sh[j * nbw + (hx >> 5)] >> (hx & 31)) & 1;
                        const uint32_t col = side * job.side_pad + h;
                        const uint32_t gb = (grow[col >> 5] >> (col & 31)) & 1;
                        fc = !pat;
                        composite = (sb | gb) != 0;
                    }
                    const uint32_t fcm = __ballot_sync(0xFFFFFFFFu, fc);
                    const uint32_t cm = __ballot_sync(0xFFFFFFFFu, composite);
                    unk += __popc(fcm & ~cm);
                    if (lane == 0) {
                        uint32_t m = fcm;
                        while (m) {
                            const uint32_t i = __ffs(m) - 1;
                            m &= m - 1;
                            b |= ((cm >> i) & 1u) << bit;
                            if (++bit == 7) {
                                bytes[nbytes++] = (uint8_t)b;
                                b = 0x80;
                                bit = 0;
                            }
                        }
                    }
                }
            }
            if (lane == 0) {
                if (bit) bytes[nbytes++] = (uint8_t)b;
                rd.counts[2 * row] = unk;
                rd.counts[2 * row + 1] = nbytes;
                const uint64_t m = job.mstart + s_mi[j];
                // "m : U B || <bytes>\n"
                rd.row_bytes[row] = ndigits(m) + ndigits(unk) + ndigits(nbytes) + 9 + nbytes;
            }
        }
        return;
    }
    // Plain and RLE rows.  The large-prime marks (one bit per live offset,
    // in distance order on each side) go into the row's bitmap over offset
    // indexes, one lane per word of marks; then the live offsets left
    // unmarked are read off that bitmap a word per lane, nearest to SL first
    // on each side, each distance following from its index.
    const uint32_t side_words = job.side_pad >> 5;
    const uint32_t hs = (sl - x_par + 1) >> 1;  // indexes below hs: x < SL
    for (uint32_t j = warp; j < nrows; j += nwarps) {
        const uint32_t row = r0 + j;
        const uint32_t *grow = job.comp + (uint64_t)row * job.pitch;
        uint32_t *bm = sh + j * nbw;
        for (uint32_t cw = lane; cw < 2 * side_words; cw += 32) {
            uint32_t bits = grow[cw];
            const uint32_t side = cw >= side_words ? 1u : 0u;
            const uint32_t h0 = 32 * (cw - side * side_words);
            while (bits) {
                const uint32_t h = h0 + __ffs(bits) - 1;
                bits &= bits - 1;
                if (h >= H) continue;  // columns past H are never marked
                const uint32_t d = rd.dist[h];
                const uint32_t hx = ((side ? sl + d : sl - d) - x_par) >> 1;
                atomicOr(&bm[hx >> 5], 1u << (hx & 31));
            }
        }
        __syncwarp();
        uint32_t *list = rd.lists + (uint64_t)row * 2 * H;
        uint64_t body = 0;
        uint32_t cnt_side[2];
        for (uint32_t side = 0; side < 2; side++) {
            // side 1: words from hs / 32 up; side 0: from (hs - 1) / 32 down
            const uint32_t first = side ? hs >> 5 : (hs ? (hs - 1) >> 5 : 0);
            const uint32_t nw = side ? nbw - (hs >> 5) : (hs ? ((hs - 1) >> 5) + 1 : 0);
            uint32_t *out = list + side * H;
            uint32_t cnt = 0, dsum = 0;
            for (uint32_t k0 = 0; k0 < nw; k0 += 32) {
                const uint32_t k = k0 + lane;
                uint32_t u = 0, w = 0;
                if (k < nw) {
                    w = side ? first + k : first - k;
                    u = rd.live[w] & ~bm[w];
                    // the word holding hs has indexes of both sides
                    const uint32_t lo = 32 * w;
                    if (side) {
                        if (lo < hs) u &= ~0u << (hs - lo);
                    } else if (lo + 32 > hs) {
                        u &= (1u << (hs - lo)) - 1;
                    }
                }
                const uint32_t c = __popc(u);
                uint32_t incl = c;
#pragma unroll
                for (uint32_t off = 1; off < 32; off <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, off);
                    if ((uint32_t)lane >= off) incl += t;
                }
                uint32_t idx = cnt + incl - c;
                // distances ascend within the word: D digits below T = 10^D
                // (64-bit: the loop below ends for any 32-bit distance)
                uint32_t D = 0;
                uint64_t T = 1;
                while (u) {
                    const uint32_t b = side ? __ffs(u) - 1 : 31 - __clz(u);
                    u ^= 1u << b;
                    const uint32_t x = 2 * (32 * w + b) + x_par;
                    const uint32_t d = side ? x - sl : sl - x;
                    out[idx++] = d;
                    while (d >= T) {
                        D++;
                        T *= 10;
                    }
                    dsum += D;
                }
                cnt += __shfl_sync(0xFFFFFFFFu, incl, 31);
            }
            dsum = __reduce_add_sync(0xFFFFFFFFu, dsum);
            cnt_side[side] = cnt;
            body += dsum;
        }
        if (lane == 0) {
            rd.counts[2 * row] = cnt_side[0];
            rd.counts[2 * row + 1] = cnt_side[1];
            uint64_t m = job.mstart + s_mi[j];
            uint64_t n = cnt_side[0] + (uint64_t)cnt_side[1];
            uint64_t bytes = ndigits(m) + ndigits(cnt_side[0]) + ndigits(cnt_side[1]);
            if (rd.compression == 1) bytes += 13 + 2 * n;
            else bytes += 11 + 2 * n + body;
            rd.row_bytes[row] = bytes;
        }
    }
}

// ---- exclusive scan of u64 (three passes) -----------------------------------

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint64_t kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ uint64_t warp_incl_scan(uint64_t v) {
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total
__device__ uint64_t block_excl_scan(uint64_t v, uint64_t &excl) {
    __shared__ uint64_t s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t incl = warp_incl_scan(v);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
        w = warp_incl_scan(w);
        s_warp[lane] = w;
    }
    __syncthreads();
    uint64_t before = warp > 0 ? s_warp[warp - 1] : 0;
    excl = before + incl - v;
    uint64_t total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint64_t *in, uint64_t n,
                                                                   uint64_t *block_sums) {
    uint64_t base = (uint64_t)blockIdx.x * kScanChunk;
    uint64_t s = 0;
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + (uint64_t)threadIdx.x * kScanItems + k;
        if (i < n) s += in[i];
    }
    uint64_t excl;
    uint64_t total = block_excl_scan(s, excl);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(uint64_t *block_sums, uint64_t nb,
                                                                   uint64_t *total, const uint64_t *base) {
    __shared__ uint64_t s_carry;
    if (threadIdx.x == 0) s_carry = base ? *base : 0;
    __syncthreads();
    for (uint64_t b0 = 0; b0 < nb; b0 += kScanThreads) {
        uint64_t i = b0 + threadIdx.x;
        uint64_t v = i < nb ? block_sums[i] : 0;
        uint64_t excl;
        uint64_t t = block_excl_scan(v, excl);
        if (i < nb) block_sums[i] = s_carry + excl;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += t;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint64_t *in, uint64_t n,
                                                                  const uint64_t *block_sums,
                                                                  uint64_t *out) {
    uint64_t base = (uint64_t)blockIdx.x * kScanChunk;
    uint64_t vals[kScanItems];
    uint64_t s = 0;
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + (uint64_t)threadIdx.x * kScanItems + k;
        vals[k] = i < n ? in[i] : 0;
        s += vals[k];
    }
    uint64_t excl;
    block_excl_scan(s, excl);
    uint64_t run = block_sums[blockIdx.x] + excl;
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + (uint64_t)threadIdx.x * kScanItems + k;
        if (i < n) out[i] = run;
        run += vals[k];
    }
}

// ---- text -----------------------------------------------------------------------

__device__ __forceinline__ uint32_t put_u64(char *dst, uint64_t v) {
    char t[20];
    uint32_t n = 0;
    do {
        t[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    for (uint32_t i = 0; i < n; i++) dst[i] = t[n - 1 - i];
    return n;
}

// One warp per row.  Plain rows: "m : -nl +nh | -d1 -d2 | +d1 +d2\n"
// (combined_sieve.cpp:1387-1438); RLE rows encode each distance step as two
// characters 48 + (delta >> 7), 48 + (delta & 127) (combined_sieve.cpp:1396-1417).
__global__ void __launch_bounds__(256) format_kernel(RowsDev rd, const uint64_t *offsets, char *text,
                                                     uint32_t row_lo, uint32_t row_hi) {
    const JobDev &job = rd.job;
    const uint32_t row = row_lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= row_hi) return;
    const uint32_t H = job.half_cols;
    const uint32_t *list = rd.lists + (uint64_t)row * 2 * H;
    const uint32_t cnt[2] = {rd.counts[2 * row], rd.counts[2 * row + 1]};
    // a row whose bytes would not fit is skipped (the host then sees a total
    // above the capacity and reports an error); never reached with exact counts
    if (offsets[row] + rd.row_bytes[row] > rd.text_cap) return;
    char *out = text + offsets[row];
    uint64_t pos = 0;
    if (rd.compression == 2) {
        const uint64_t m = job.mstart + rd.valid_mi[row];
        if (lane == 0) {
            pos += put_u64(out + pos, m);
            out[pos++] = ' ';
            out[pos++] = ':';
            out[pos++] = ' ';
            pos += put_u64(out + pos, cnt[0]);
            out[pos++] = ' ';
            pos += put_u64(out + pos, cnt[1]);
            out[pos++] = ' ';
            out[pos++] = '|';
            out[pos++] = '|';
            out[pos++] = ' ';
        }
        pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
        const uint8_t *bytes = (const uint8_t *)list;
        for (uint32_t i = lane; i < cnt[1]; i += 32) out[pos + i] = (char)bytes[i];
        if (lane == 0) out[pos + cnt[1]] = '\n';
        return;
    }
    if (lane == 0) {
        uint64_t m = job.mstart + rd.valid_mi[row];
        pos += put_u64(out + pos, m);
        out[pos++] = ' ';
        out[pos++] = ':';
        out[pos++] = ' ';
        out[pos++] = '-';
        pos += put_u64(out + pos, cnt[0]);
        out[pos++] = ' ';
        out[pos++] = '+';
        pos += put_u64(out + pos, cnt[1]);
        out[pos++] = ' ';
    }
    pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
    const bool rle = rd.compression == 1;
    for (uint32_t side = 0; side < 2; side++) {
        if (lane == 0) {
            out[pos] = '|';
            if (rle) out[pos + 1] = ' ';
        }
        pos += rle ? 2 : 1;
        const char sign = side ? '+' : '-';
        for (uint32_t i0 = 0; i0 < cnt[side]; i0 += 32) {
            uint32_t i = i0 + lane;
            bool on = i < cnt[side];
            uint32_t d = on ? list[side * H + i] : 0;
            uint32_t len = 0;
            if (on) {
                if (rle) len = 2;
                else len = 2 + ndigits(d);
            }
            uint32_t incl = len;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += t;
            }
            if (on) {
                char *dst = out + pos + (incl - len);
                if (rle) {
                    uint32_t prev = i == 0 ? 0 : list[side * H + i - 1];
                    uint32_t delta = d - prev;
                    dst[0] = (char)(unsigned char)(48 + (delta >> 7));
                    dst[1] = (char)(unsigned char)(48 + (delta & 127));
                } else {
                    dst[0] = ' ';
                    dst[1] = sign;
                    put_u64(dst + 2, d);
                }
            }
            pos += __shfl_sync(0xFFFFFFFFu, incl, 31);
        }
        if (lane == 0) out[pos] = side ? '\n' : ' ';
        pos += 1;
    }
}

}  // namespace

cudaError_t rows_extract(const RowsDev &rd, uint32_t rows_per_block, cudaStream_t stream, uint32_t row_lo,
                         uint32_t row_hi) {
    row_hi = std::min(row_hi, (uint32_t)rd.job.rows);
    if (row_lo >= row_hi) return cudaSuccess;
    if (row_lo % rows_per_block) return cudaErrorInvalidValue;
    if (rd.nd > (uint32_t)kMaxDPrimes) return cudaErrorInvalidValue;
    const uint32_t nbw = (rd.nb + 31) / 32;
    size_t smem = ((size_t)rows_per_block * nbw * (rd.compression == 2 ? 2 : 1) + rows_per_block +
                   (size_t)rows_per_block * kMaxDPrimes) * sizeof(uint32_t);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e) return e;
    }
    uint32_t blocks = (row_hi - row_lo + rows_per_block - 1) / rows_per_block;
    rows_kernel<<<blocks, kRowThreads, smem, stream>>>(rd, rows_per_block, row_lo / rows_per_block);
    return cudaGetLastError();
}

uint64_t scan_tmp_words(uint64_t n) { return (n + kScanChunk - 1) / kScanChunk + 1; }

cudaError_t scan_u64(const uint64_t *d_in, uint64_t *d_out, uint64_t *d_total, uint64_t n,
                     uint64_t *d_tmp, cudaStream_t stream, const uint64_t *d_base) {
    if (n == 0) {
        if (d_base) return cudaMemcpyAsync(d_total, d_base, sizeof(uint64_t), cudaMemcpyDeviceToDevice, stream);
        return cudaMemsetAsync(d_total, 0, sizeof(uint64_t), stream);
    }
    uint64_t nb = (n + kScanChunk - 1) / kScanChunk;
    scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(d_in, n, d_tmp);
    scan_blocks_kernel<<<1, kScanThreads, 0, stream>>>(d_tmp, nb, d_total, d_base);
    scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(d_in, n, d_tmp, d_out);
    return cudaGetLastError();
}

cudaError_t format_rows(const RowsDev &rd, const uint64_t *d_offsets, char *d_text, cudaStream_t stream,
                        uint32_t row_lo, uint32_t row_hi) {
    row_hi = std::min(row_hi, (uint32_t)rd.job.rows);
    if (row_lo >= row_hi) return cudaSuccess;
    uint64_t threads = (uint64_t)(row_hi - row_lo) * 32;
    format_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, stream>>>(rd, d_offsets, d_text, row_lo,
                                                                          row_hi);
    return cudaGetLastError();
}

}  // namespace pg
