// Host-side job derivation and buffer helpers of libpgsieve (see pg_host.h).
//
// A job's tables follow prime_gap_parallel's setup (combined_sieve.cpp:2014-2200):
// validation (gap_common.cpp:1007-1094, combined_sieve.cpp:86-135),
// K = P#/d (gap_common.cpp:116-121), valid m (gap_common.cpp:307-342),
// offsets coprime to K (combined_sieve.cpp:1143-1169) and the thresholds of
// calculate_thresholds_method2 (gap_common.cpp:345-375).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "pg_host.h"
#include "pg_tuning.h"

namespace pgh {

bool is_prime_u64(uint64_t n) {
    if (n < 2) return false;
    if (n % 2 == 0) return n == 2;
    for (uint64_t t = 3; t * t <= n; t += 2)
        if (n % t == 0) return false;
    return true;
}

uint64_t next_prime_above(uint64_t n) {
    uint64_t c = n + 1;
    while (!is_prime_u64(c)) c++;
    return c;
}

std::vector<uint32_t> primes_upto(uint32_t n) {
    std::vector<uint32_t> out;
    if (n < 2) return out;
    std::vector<uint8_t> comp(n + 1, 0);
    for (uint32_t i = 2; i <= n; i++) {
        if (comp[i]) continue;
        out.push_back(i);
        for (uint64_t j = (uint64_t)i * i; j <= n; j += i) comp[j] = 1;
    }
    return out;
}

uint32_t ndigits(uint64_t v) {
    uint32_t n = 1;
    while (v >= 10) v /= 10, n++;
    return n;
}

// A bitmask as {bits, rank} pairs: word w of the mask followed by the number
// of set bits in words [0, w), so that the rank of any bit is one pair read
// and a popcount.
static std::vector<uint32_t> with_ranks(const std::vector<uint32_t> &mask) {
    std::vector<uint32_t> out(2 * mask.size());
    uint32_t run = 0;
    for (size_t w = 0; w < mask.size(); w++) {
        out[2 * w] = mask[w];
        out[2 * w + 1] = run;
        run += (uint32_t)__builtin_popcount(mask[w]);
    }
    return out;
}

int derive(const pgs_job &j, HostJob &h, std::string &err, bool tables) {
    h.job = j;
    // Args::argparse validation (gap_common.cpp:1007-1094)
    if (j.p < 2) {
        err = "p must be a prime >= 2";
        return PGS_EABORT;  // get_sieve_primes(P).back() == P asserts
    }
    if (j.p >= 10000000u || !is_prime_u64(j.p)) {
        err = "p# not prime";
        return PGS_EINVAL;
    }
    if (j.mstart == 0) return err = "mstart must be greater than 0", PGS_EINVAL;
    if (j.minc == 0) return err = "minc must be greater than 0", PGS_EINVAL;
    if (j.minc >= 0x7FFFFFFFull) return err = "minc must be less than 2B", PGS_EINVAL;
    if (j.mstart + j.minc > 10000000001ull) return err = "mstart + minc must be <= 10e9", PGS_EINVAL;
    if (j.max_prime > 40000000000000ull) return err = "max_prime > 40 Trillion not supported", PGS_EINVAL;
    if (j.max_prime < 3) return err = "max_prime must be set", PGS_EINVAL;
    if (j.d == 0) return err = "d must be greater than 0", PGS_EINVAL;
    if (j.compression < 0 || j.compression > 2) return err = "unknown compression", PGS_EINVAL;
    const uint32_t P = j.p, D = j.d, SL = j.sieve_length;
    std::vector<uint32_t> pp = primes_upto(P);
    if (SL % 500 != 0) {
        for (uint32_t q : pp) {
            if (q >= P) break;
            if (SL % q == 0 && D % q != 0) return err = "SL not coprime", PGS_EINVAL;
        }
    }
    // combined_sieve.cpp:97-103
    if ((uint64_t)SL < 6ull * P || (uint64_t)SL > 22ull * P)
        return err = "sieve_length outside [6P, 22P]", PGS_EINVAL;
    if (2ull * SL + 1 > 4000000ull) return err = "sieve_length too large (2*SL+1 above 4,000,000)", PGS_EINVAL;

    // K = P#/d (gap_common.cpp:116-121); d must divide P#
    {
        uint32_t rest = D;
        std::vector<uint32_t> limbs{1};
        for (uint32_t q : pp) {
            if (rest % q == 0) {
                rest /= q;
                if (q != 2) h.dq.push_back(q);
                continue;
            }
            uint64_t carry = 0;
            for (auto &l : limbs) {
                uint64_t t = (uint64_t)l * q + carry;
                l = (uint32_t)t;
                carry = t >> 32;
            }
            if (carry) limbs.push_back((uint32_t)carry);
        }
        if (rest != 1) return err = "d does not divide P#", PGS_EABORT;
        if (limbs.size() == 1 && limbs[0] <= 1) return err = "K <= 1", PGS_EABORT;
        h.klimbs = limbs;
        h.kbits = 32 * (uint32_t)(limbs.size() - 1) + (32 - __builtin_clz(limbs.back()));
    }
    const bool d_even = (D % 2) == 0;
    h.x_par = d_even ? (SL & 1) : ((SL + 1) & 1);
    h.nb = h.x_par == 0 ? SL + 1 : SL;

    // valid m (gap_common.cpp:307-342).  The m and offset flags live in
    // per-thread scratch that keeps its pages from one job to the next.
    const uint64_t minc = j.minc, ms = j.mstart;
    static thread_local std::vector<uint8_t> m_ok, coprime;
    struct Trim {  // a huge job's flags are not kept past the call
        ~Trim() {
            for (std::vector<uint8_t> *v : {&m_ok, &coprime})
                if (v->capacity() > (16u << 20)) std::vector<uint8_t>().swap(*v);
        }
    } trim;
    m_ok.assign(minc, 1);
    for (uint32_t q : pp) {
        if (D % q) continue;
        uint64_t first = (q - (ms % q)) % q;
        for (uint64_t mi = first; mi < minc; mi += q) m_ok[mi] = 0;
    }
    uint64_t valid = 0;
    {
        const uint8_t *f = m_ok.data();
        uint32_t acc = 0;  // minc < 2^31
        for (uint64_t mi = 0; mi < minc; mi++) acc += f[mi];
        valid = acc;
    }
    if (valid == 0) return err = "no m coprime to d", PGS_EABORT;

    // offsets coprime to K (combined_sieve.cpp:1143-1169)
    const uint32_t interval = 2 * SL + 1;
    coprime.assign(interval, 1);
    for (uint32_t q : pp) {
        if (D % q == 0) continue;
        for (uint32_t x = SL % q; x < interval; x += q) coprime[x] = 0;
    }
    uint64_t cc = 0;
    for (uint32_t x = 0; x < interval; x++) cc += coprime[x];
    h.coprime_x = cc;

    // calculate_thresholds_method2 (gap_common.cpp:345-375), same conversions
    {
        uint32_t sieve_interval = interval;
        double sm = std::log(8.0) * (double)minc / (double)valid;
        float SMALL_MULT = (float)(8.0 > sm ? 8.0 : sm);
        uint64_t MEDIUM_CROSSOVER_SMALL = (uint64_t)(1.0 * (double)cc * (double)minc / (double)valid);
        float M_PER_P_CROSSOVER = (float)(1.0 * (double)minc * sieve_interval / (double)cc);
        double mm = 0.65 * std::log2((double)(M_PER_P_CROSSOVER / (float)cc));
        float MEDIUM_MULT = (float)(1.9 > mm ? 1.9 : mm);
        uint64_t MEDIUM_CROSSOVER_SEARCH = (uint64_t)(MEDIUM_MULT * M_PER_P_CROSSOVER);
        uint64_t SMALL = (uint64_t)SMALL_MULT * sieve_interval;
        if (MEDIUM_CROSSOVER_SMALL < SMALL) SMALL = MEDIUM_CROSSOVER_SMALL;
        if (SMALL < sieve_interval) SMALL = sieve_interval + 1;
        uint64_t MEDIUM = SMALL > MEDIUM_CROSSOVER_SEARCH ? SMALL : MEDIUM_CROSSOVER_SEARCH;
        if (MEDIUM > j.max_prime) MEDIUM = j.max_prime;
        h.small_threshold = SMALL;
        h.medium_threshold = MEDIUM;
        // combined_sieve.cpp:2080-2082 asserts MEDIUM >= SMALL
        if (MEDIUM < SMALL) return err = "MEDIUM_THRESHOLD < SMALL_THRESHOLD", PGS_EABORT;
    }
    // Primes sieved by the reference: all primes < max_prime, and the small
    // phase runs through the first prime above SMALL_THRESHOLD
    // (combined_sieve.cpp:1481-1504).
    {
        uint64_t small_last = next_prime_above(h.small_threshold);
        h.prime_limit = std::max<uint64_t>(j.max_prime - 1, small_last);
    }
    h.s1 = 4ull * SL + 2;
    for (uint32_t q : pp)
        if (q <= h.prime_limit) h.primes_to_P++;

    char fn[256];
    snprintf(fn, sizeof fn, "unknowns/%u_%u_%llu_%llu_s%u_l%lluM.txt", P, D,
             (unsigned long long)ms, (unsigned long long)minc, SL,
             (unsigned long long)(j.max_prime / 1000000ull));
    h.filename = fn;
    if (!tables) return PGS_OK;

    // lists written without branches: every index is stored, and the
    // write position advances past the ones that stay
    h.valid_mi.resize(valid + 1);
    {
        uint32_t *o = h.valid_mi.data();
        uint64_t n = 0;
        for (uint64_t mi = 0; mi < minc; mi++) {
            o[n] = (uint32_t)mi;
            n += m_ok[mi];
        }
    }
    h.valid_mi.resize(valid);
    // live offsets: coprime to K and of the parity that makes m*K + X odd
    {
        const uint32_t dd0 = ((SL + 1) & 1) == h.x_par ? 1 : 2;
        h.dist.resize(SL / 2 + 2);
        uint32_t *o = h.dist.data();
        uint32_t n = 0;
        for (uint32_t dd = dd0; dd <= SL; dd += 2) {
            o[n] = dd;
            n += coprime[SL + dd];
        }
        h.dist.resize(n);
    }
    h.H = (uint32_t)h.dist.size();
    h.live.assign((h.nb + 31) / 32, 0);
    for (uint32_t dd : h.dist)
        for (uint32_t x : {SL - dd, SL + dd}) {
            const uint32_t hx = (x - h.x_par) >> 1;
            h.live[hx >> 5] |= 1u << (hx & 31);
        }
    h.Hp = (h.H + 31) / 32 * 32;
    h.pitch = (2 * h.Hp / 32 + 3) / 4 * 4;
    if (h.pitch == 0) h.pitch = 4;
    // parity-reduced large-prime walk (pg::WalkParams)
    pg::WalkParams &w = h.walk;
    if (d_even) {
        w.stride = 2;
        w.mi_base = (ms & 1) ? 0 : 1;  // valid m are odd
        w.jmax = minc > w.mi_base ? (minc - w.mi_base + 1) / 2 : 0;
        w.c_add = SL / 2;
        w.w = 2 * (SL / 2) + 1;
        w.xc = 2 * (SL / 2) + SL;
        w.odd_d = 0;
    } else {
        const uint32_t hi = (SL - 1) / 2, lo = (SL + 1) / 2;  // X' in [-lo, hi]
        w.stride = 1;
        w.mi_base = 0;
        w.jmax = minc;
        w.c_add = hi;
        w.w = hi + lo + 1;
        w.xc = 2 * hi + 1 + SL;
        w.odd_d = 1;
    }
    w.m0 = ms + w.mi_base;
    // Bitmasks over the walk's own coordinates: valid m over walk indices j
    // (mi = mi_base + stride*j; with d even every valid m is odd, on that
    // lattice) and live offsets over walk residues y (x = X + SL = xc - 2y,
    // the walk's parity of x).  A hit's bitset row is the rank of j among the
    // valid m; its column, with ry = live y below y (live x above x), is
    // ry - H for x < SL (the low side runs in distance order) and Hp+H-1-ry
    // above SL.
    h.mmask.assign((w.jmax + 31) / 32, 0);
    uint64_t on_lattice = 0;
    {
        // a word at a time in a register (mi_base + stride * j < minc)
        const uint8_t *f = m_ok.data() + w.mi_base;
        for (uint64_t wi = 0; wi < h.mmask.size(); wi++) {
            const uint64_t j0 = 32 * wi, jn = std::min<uint64_t>(32, w.jmax - j0);
            uint32_t word = 0;
            for (uint64_t b = 0; b < jn; b++) word |= (uint32_t)f[w.stride * (j0 + b)] << b;
            h.mmask[wi] = word;
            on_lattice += (uint64_t)__builtin_popcount(word);
        }
    }
    if (on_lattice != valid) return err = "valid m off the walk lattice", PGS_EABORT;
    h.ymask.assign((w.w + 31) / 32, 0);
    for (uint32_t dd : h.dist)
        for (uint32_t x : {SL - dd, SL + dd}) {
            const uint32_t y = (w.xc - x) / 2;
            h.ymask[y >> 5] |= 1u << (y & 31);
        }
    h.y_lo = (w.xc - SL) / 2 + 1;  // x < SL exactly for y >= y_lo
    h.mmask = with_ranks(h.mmask);
    h.ymask = with_ranks(h.ymask);
    return PGS_OK;
}

PinnedPool &pinned_pool() {
    static PinnedPool *pool = new PinnedPool();  // lives until exit
    return *pool;
}

int fail(pgs_ctx *ctx, cudaError_t e, const char *what) {
    if (ctx) {
        ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    if (e == cudaErrorMemoryAllocation) return PGS_ENOMEM;
    return PGS_ECUDA;
}

pg::JobDev job_dev(pgs_prepared *pr) {
    const HostJob &h = pr->hj;
    pg::JobDev j{};
    j.mstart = h.job.mstart;
    j.minc = (uint32_t)h.job.minc;
    j.sl = h.job.sieve_length;
    j.two_sl = 2 * h.job.sieve_length;
    j.rows = (uint32_t)h.valid_mi.size();
    j.half_cols = h.H;
    j.side_pad = h.Hp;
    j.pitch = h.pitch;
    j.comp = pr->comp.as<uint32_t>();
    j.y_lo = h.y_lo;
    j.walk = h.walk;
    j.kmul = 1;
    j.direct_steps = pr->tune.direct_steps;
    j.item_shift = (uint32_t)pgt::ilog2(pr->tune.item_steps);
    j.heavy_steps = pr->tune.heavy_steps;
    j.large_form = pr->tune.large_form;
    return j;
}

pg::RowsDev rows_dev(pgs_prepared *pr) {
    const HostJob &h = pr->hj;
    pg::RowsDev rd{};
    rd.job = job_dev(pr);
    rd.x_par = h.x_par;
    rd.nb = h.nb;
    rd.valid_mi = pr->valid_mi.as<uint32_t>();
    rd.dist = pr->dist.as<uint32_t>();
    rd.live = pr->live.as<uint32_t>();
    rd.nd = (uint32_t)h.dq.size();
    rd.dq = pr->dq.as<uint32_t>();
    rd.dr = pr->dr.as<uint32_t>();
    rd.sp_base = (uint32_t)pr->sp_lo;
    rd.sp = pr->sp.as<uint32_t>();
    rd.sr = pr->sr.as<uint32_t>();
    rd.sp_range = pr->misc.as<unsigned long long>() + 1;
    rd.sp_cap = pr->sp_bound;
    rd.text_cap = pr->text_cap;
    rd.lists = pr->lists.as<uint32_t>();
    rd.counts = pr->counts.as<uint32_t>();
    rd.row_bytes = pr->row_bytes.as<uint64_t>();
    rd.compression = h.job.compression;
    return rd;
}

// Rows per CTA of rows_kernel: as many as keep four 512-thread CTAs (2048
// threads, the SM's limit) resident, with their bitmaps in shared memory
// (55 KiB each), and at most `cap` (the job's tuning, 16 by default).
// SL = 2e4 (626 bitmap words per row): 16 rows run 12 % faster than 32 rows
// at two CTAs per SM.  A cap above 16 trades resident CTAs for rows: up to
// the 220 KiB a CTA may hold.
uint32_t rows_per_block(uint32_t nb, int compression, uint32_t cap) {
    const uint32_t nbw = (nb + 31) / 32;
    const uint32_t per_row = nbw * 4u * (compression == 2 ? 2u : 1u) + 4u + 64u;
    uint32_t r = (cap > 16 ? 225280u : 56320u) / per_row;
    if (r > cap) r = cap;
    if (r < 1) r = 1;
    return r;
}

cudaError_t upload_tables(pgs_prepared *pr, cudaStream_t s) {
    const HostJob &h = pr->hj;
    struct Item {
        DevBuf *b;
        const void *src;
        size_t n;
    } items[] = {{&pr->klimbs, h.klimbs.data(), h.klimbs.size() * 4},
                 {&pr->valid_mi, h.valid_mi.data(), h.valid_mi.size() * 4},
                 {&pr->dist, h.dist.data(), h.dist.size() * 4},
                 {&pr->live, h.live.data(), h.live.size() * 4},
                 {&pr->dq, h.dq.data(), h.dq.size() * 4},
                 {&pr->mmask, h.mmask.data(), h.mmask.size() * 4},
                 {&pr->ymask, h.ymask.data(), h.ymask.size() * 4}};
    size_t total = 0;
    for (const Item &it : items) total += (it.n + 255) / 256 * 256;
    if (!pr->stage || pr->stage_cap < total) {
        if (pr->stage) pinned_pool().put(pr->stage, pr->stage_cap);
        pr->stage = pinned_pool().get(total + 256, &pr->stage_cap);
        if (!pr->stage) return cudaErrorMemoryAllocation;
    }
    size_t off = 0;
    for (const Item &it : items) {
        cudaError_t e = it.b->ensure(it.n);
        if (e) return e;
        if (it.n) {
            memcpy(pr->stage + off, it.src, it.n);
            e = cudaMemcpyAsync(it.b->p, pr->stage + off, it.n, cudaMemcpyHostToDevice, s);
            if (e) return e;
        }
        off += (it.n + 255) / 256 * 256;
    }
    return cudaSuccess;
}

size_t job_ranges(const pgs_prepared *pr) {
    return 1 + (pr->table_mode ? pr->tbl_windows.size() : pr->windows.size());
}

int fetch_job(pgs_ctx *ctx, pgs_prepared *pr, cudaStream_t s, pgs_result *out, const HostText *given) {
    memset(out, 0, sizeof(*out));
    const HostJob &h = pr->hj;
    // misc: [0] text bytes, then {begin, end} pairs: small primes, then windows
    const size_t nr = job_ranges(pr);
    std::vector<uint64_t> misc(1 + 2 * nr);
    CK(cudaMemcpyAsync(misc.data(), pr->misc.p, misc.size() * 8, cudaMemcpyDeviceToHost, s));
    // per-row unknown counts: their sum is the result's total
    std::vector<uint32_t> counts(2 * h.valid_mi.size());
    if (!counts.empty())
        CK(cudaMemcpyAsync(counts.data(), pr->counts.p, counts.size() * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint64_t total = given ? given->total : misc[0];
    if (total > pr->text_cap) {
        ctx->err = "text larger than its bound";
        return PGS_ECUDA;
    }
    size_t cap = 0;
    char *host = nullptr;
    float ms_d2h = 0;
    if (given) {
        host = given->text;
        cap = given->cap;
        ms_d2h = given->ms_d2h;
    } else {
        host = pinned_pool().get(total + 1, &cap);
        if (!host) {
            ctx->err = "cudaMallocHost failed";
            return PGS_ENOMEM;
        }
        cudaEvent_t t0, t1;
        CK(cudaEventCreate(&t0));
        CK(cudaEventCreate(&t1));
        CK(cudaEventRecord(t0, s));
        if (total) CK(cudaMemcpyAsync(host, pr->text.p, total, cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(t1, s));
        CK(cudaStreamSynchronize(s));
        host[total] = 0;
        cudaEventElapsedTime(&ms_d2h, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }

    out->text = host;
    out->text_len = total;
    out->internal = new PinnedOwner{cap};
    out->rows = h.valid_mi.size();
    // (low, high) per row; bitcompressed rows keep (unknowns, bytes)
    uint64_t unknowns = 0;
    const size_t step = h.job.compression == 2 ? 2 : 1;
    for (size_t i = 0; i < counts.size(); i += step) unknowns += counts[i];
    out->unknowns = unknowns;
    uint64_t primes = h.primes_to_P;
    if (pr->large_primes != ~0ull)
        primes += misc[2] - misc[1] + pr->large_primes;  // small-prime range, then the host's count
    else
        for (size_t i = 0; i < nr; i++) primes += misc[2 + 2 * i] - misc[1 + 2 * i];
    out->primes = primes;
    out->prime_limit = h.prime_limit;
    out->launches = pr->launches;
    out->ms_stage[PGS_STAGE_SETUP] = pr->ms_setup;
    out->ms_stage[PGS_STAGE_D2H] = ms_d2h;
    for (auto &sp : pr->spans) {
        float ms = 0;
        if (sp.second.first < 0 || sp.second.second < 0) continue;
        cudaEventElapsedTime(&ms, pr->events[sp.second.first], pr->events[sp.second.second]);
        if (sp.first < 0) out->ms_total = ms;
        else out->ms_stage[sp.first] += ms;
    }
    return PGS_OK;
}

}  // namespace pgh
