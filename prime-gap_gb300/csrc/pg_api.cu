// C ABI of libpgsieve and the host-side orchestration of one method2 job.
//
// A job follows prime_gap_parallel (combined_sieve.cpp:2014-2447):
//   host:   validation (gap_common.cpp:1007-1094, combined_sieve.cpp:86-135),
//           K = P#/d (gap_common.cpp:116-121), valid m (gap_common.cpp:307-342),
//           offsets coprime to K (combined_sieve.cpp:1143-1169), thresholds
//           (gap_common.cpp:345-375) -> small tables uploaded once;
//   device: small-prime window sieve + K mod p, then for each 2^30-wide
//           window of larger primes: sieve -> K mod p -> large-prime marks;
//           then the row phase, a prefix sum and the text of every row.
// Everything after the table upload is asynchronous on one stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pg_internal.h"
#include "pgsieve.h"

namespace {

constexpr uint64_t kWindowSpan = 1ull << 30;

// ---------------------------------------------------------------------------
// host number theory for job setup

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

struct HostJob {
    pgs_job job{};
    std::vector<uint32_t> klimbs;
    uint32_t kbits = 0;
    std::vector<uint32_t> valid_mi;
    std::vector<int32_t> row_of_mi;
    std::vector<int32_t> col_of_x;
    std::vector<uint32_t> dist;
    std::vector<uint32_t> dq;  // odd primes dividing d
    std::vector<uint32_t> mmask, xmask;  // valid-m and live-offset bitmasks
    uint32_t x_par = 0, nb = 0, H = 0, Hp = 0, pitch = 0;
    uint64_t coprime_x = 0;
    uint64_t small_threshold = 0, medium_threshold = 0, prime_limit = 0;
    uint64_t s1 = 0;
    uint64_t primes_to_P = 0;  // primes <= min(P, prime_limit), 2 included
    pg::WalkParams walk{};
    std::string filename;
};

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
    if (2ull * SL + 1 > 4000000ull) return err = "sieve_length too large for this build", PGS_EINVAL;

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

    // valid m (gap_common.cpp:307-342)
    const uint64_t minc = j.minc, ms = j.mstart;
    std::vector<uint8_t> m_ok(minc, 1);
    for (uint32_t q : pp) {
        if (D % q) continue;
        uint64_t first = (q - (ms % q)) % q;
        for (uint64_t mi = first; mi < minc; mi += q) m_ok[mi] = 0;
    }
    uint64_t valid = 0;
    for (uint64_t mi = 0; mi < minc; mi++) valid += m_ok[mi];
    if (valid == 0) return err = "no m coprime to d", PGS_EABORT;

    // offsets coprime to K (combined_sieve.cpp:1143-1169)
    const uint32_t interval = 2 * SL + 1;
    std::vector<uint8_t> coprime(interval, 1);
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

    h.valid_mi.reserve(valid);
    h.row_of_mi.assign(minc, -1);
    for (uint64_t mi = 0; mi < minc; mi++) {
        if (m_ok[mi]) {
            h.row_of_mi[mi] = (int32_t)h.valid_mi.size();
            h.valid_mi.push_back((uint32_t)mi);
        }
    }
    // live offsets: coprime to K and of the parity that makes m*K + X odd
    for (uint32_t dd = 1; dd <= SL; dd++) {
        uint32_t x = SL + dd;
        if (coprime[x] && ((x & 1) == h.x_par)) h.dist.push_back(dd);
    }
    h.H = (uint32_t)h.dist.size();
    h.Hp = (h.H + 31) / 32 * 32;
    h.pitch = (2 * h.Hp / 32 + 3) / 4 * 4;
    if (h.pitch == 0) h.pitch = 4;
    h.col_of_x.assign(interval, -1);
    h.xmask.assign((interval + 31) / 32, 0);
    for (uint32_t i = 0; i < h.H; i++) {
        uint32_t lo = SL - h.dist[i], hi = SL + h.dist[i];
        h.col_of_x[lo] = (int32_t)i;
        h.col_of_x[hi] = (int32_t)(h.Hp + i);
        h.xmask[lo >> 5] |= 1u << (lo & 31);
        h.xmask[hi >> 5] |= 1u << (hi & 31);
    }
    h.mmask.assign((minc + 31) / 32, 0);
    for (uint64_t mi = 0; mi < minc; mi++)
        if (m_ok[mi]) h.mmask[mi >> 5] |= 1u << (mi & 31);
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
    return PGS_OK;
}

// ---------------------------------------------------------------------------
// device buffers and the pinned host pool

// Device allocations recycled across jobs on one context: a job's buffers
// (several GB for the larger configs) are returned here instead of freed, so
// repeated jobs pay no cudaMalloc/cudaFree.
struct DevicePool {
    std::mutex mu;
    std::vector<std::pair<void *, size_t>> free_list;
    cudaError_t get(size_t n, void **p, size_t *cap) {
        {
            std::lock_guard<std::mutex> g(mu);
            size_t best = (size_t)-1;
            for (size_t i = 0; i < free_list.size(); i++)
                if (free_list[i].second >= n &&
                    (best == (size_t)-1 || free_list[i].second < free_list[best].second))
                    best = i;
            // reuse only blocks that are not much larger than the request
            if (best != (size_t)-1 && free_list[best].second <= 2 * n + (1u << 20)) {
                *p = free_list[best].first;
                *cap = free_list[best].second;
                free_list.erase(free_list.begin() + best);
                return cudaSuccess;
            }
        }
        cudaError_t e = cudaMalloc(p, n);
        if (e == cudaErrorMemoryAllocation) {
            trim();  // give cached blocks back and retry once
            e = cudaMalloc(p, n);
        }
        if (e == cudaSuccess) *cap = n;
        return e;
    }
    void put(void *p, size_t cap) {
        std::lock_guard<std::mutex> g(mu);
        free_list.push_back({p, cap});
    }
    void trim() {
        std::lock_guard<std::mutex> g(mu);
        for (auto &b : free_list) cudaFree(b.first);
        free_list.clear();
    }
};

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    DevicePool *pool = nullptr;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= n && p) return cudaSuccess;
        release();
        size_t want = bytes < 256 ? 256 : bytes;
        if (pool) return pool->get(want, &p, &n);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() {
        if (p) {
            if (pool) pool->put(p, n);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
    template <typename T>
    T *as() const {
        return (T *)p;
    }
};

struct PinnedPool {
    std::mutex mu;
    std::vector<std::pair<char *, size_t>> free_list;
    char *get(size_t n, size_t *cap) {
        std::lock_guard<std::mutex> g(mu);
        size_t best = (size_t)-1;
        for (size_t i = 0; i < free_list.size(); i++)
            if (free_list[i].second >= n && (best == (size_t)-1 || free_list[i].second < free_list[best].second))
                best = i;
        if (best != (size_t)-1) {
            auto e = free_list[best];
            free_list.erase(free_list.begin() + best);
            *cap = e.second;
            return e.first;
        }
        char *p = nullptr;
        size_t want = n < 4096 ? 4096 : n;
        if (cudaMallocHost(&p, want) != cudaSuccess) return nullptr;
        *cap = want;
        return p;
    }
    void put(char *p, size_t cap) {
        std::lock_guard<std::mutex> g(mu);
        free_list.push_back({p, cap});
    }
};
PinnedPool &pinned_pool() {
    static PinnedPool *pool = new PinnedPool();  // lives until exit
    return *pool;
}

struct PinnedOwner {
    size_t cap;
};

struct Window {
    uint64_t lo, hi, bound;
    bool wide;
};

}  // namespace

struct pgs_ctx {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string err;
    pg::BasePrimes base;
    DevBuf win_off, win_r, win_t0, large_ctr, heavy;
    DevicePool dpool;
};

struct pgs_prepared {
    pgs_ctx *ctx = nullptr;
    HostJob hj;
    std::vector<Window> windows;
    uint64_t sp_lo = 0, sp_hi = 0, sp_bound = 0;
    uint64_t text_cap = 0;
    uint64_t win_bound = 0;
    DevBuf klimbs, row_of_mi, col_of_x, valid_mi, dist, dq, dr, comp, sp, sr, sp_t0, mmask, xmask;
    DevBuf lists, counts, row_bytes, offsets, scan_tmp, misc, text;
    std::vector<cudaEvent_t> events;
    std::vector<std::pair<int, std::pair<int, int>>> spans;  // stage, (ev a, ev b)
    double ms_setup = 0;
    uint64_t launches = 0;
    bool ran = false;
    std::vector<DevBuf *> all() {
        return {&klimbs, &row_of_mi, &col_of_x, &valid_mi, &dist,   &dq,     &dr,
                &comp,   &sp,        &sr,       &sp_t0,    &lists,  &counts, &row_bytes,
                &offsets, &scan_tmp, &misc,     &text,     &mmask,  &xmask};
    }
    ~pgs_prepared() {
        for (auto e : events) cudaEventDestroy(e);
        for (DevBuf *b : all()) b->release();
    }
};

namespace {

int fail(pgs_ctx *ctx, cudaError_t e, const char *what) {
    if (ctx) {
        ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    if (e == cudaErrorMemoryAllocation) return PGS_ENOMEM;
    return PGS_ECUDA;
}

#define CK(x)                                              \
    do {                                                   \
        cudaError_t e_ = (x);                              \
        if (e_ != cudaSuccess) return fail(ctx, e_, #x);   \
    } while (0)

template <typename T>
cudaError_t upload(DevBuf &b, const std::vector<T> &v, cudaStream_t s) {
    cudaError_t e = b.ensure(v.size() * sizeof(T));
    if (e || v.empty()) return e;
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
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
    j.row_of_mi = pr->row_of_mi.as<int32_t>();
    j.col_of_x = pr->col_of_x.as<int32_t>();
    j.comp = pr->comp.as<uint32_t>();
    j.walk = h.walk;
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
    rd.nd = (uint32_t)h.dq.size();
    rd.dq = pr->dq.as<uint32_t>();
    rd.dr = pr->dr.as<uint32_t>();
    rd.sp_base = (uint32_t)pr->sp_lo;
    rd.sp = pr->sp.as<uint32_t>();
    rd.sr = pr->sr.as<uint32_t>();
    rd.sp_count = pr->misc.as<unsigned long long>() + 1;
    rd.sp_cap = pr->sp_bound;
    rd.text_cap = pr->text_cap;
    rd.lists = pr->lists.as<uint32_t>();
    rd.counts = pr->counts.as<uint32_t>();
    rd.row_bytes = pr->row_bytes.as<uint64_t>();
    rd.compression = h.job.compression;
    return rd;
}

uint32_t rows_per_block(uint32_t nb, int compression) {
    uint32_t nbw = (nb + 31) / 32;
    uint32_t r = 98304u / (nbw * 4u * (compression == 2 ? 2u : 1u));
    if (r > 32) r = 32;
    if (r < 1) r = 1;
    return r;
}

}  // namespace

extern "C" {

const char *pgs_version(void) { return "pgsieve 0.1 (sm_103a)"; }

int pgs_create(int device, pgs_ctx **out) {
    if (!out) return PGS_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) return PGS_ENODEV;
    pgs_ctx *ctx = new pgs_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return PGS_ECUDA;
    }
    ctx->stream = ctx->own;
    *out = ctx;
    return PGS_OK;
}

void pgs_destroy(pgs_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    pg::base_primes_free(ctx->base);
    ctx->win_off.release();
    ctx->win_r.release();
    ctx->win_t0.release();
    ctx->large_ctr.release();
    ctx->heavy.release();
    ctx->dpool.trim();
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}

const char *pgs_last_error(pgs_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int pgs_set_stream(pgs_ctx *ctx, void *stream) {
    if (!ctx) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return PGS_OK;
}

void *pgs_get_stream(pgs_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int pgs_plan_job(const pgs_job *job, pgs_plan *out) {
    if (!job || !out) return PGS_EINVAL;
    HostJob h;
    std::string err;
    int rc = derive(*job, h, err, false);
    memset(out, 0, sizeof(*out));
    out->coprime_x = h.coprime_x;
    out->small_threshold = h.small_threshold;
    out->medium_threshold = h.medium_threshold;
    out->prime_limit = h.prime_limit;
    out->k_bits = h.kbits;
    snprintf(out->filename, sizeof out->filename, "%s", h.filename.c_str());
    if (rc == PGS_OK) {
        // valid m count without materialising the tables
        uint64_t valid = 0;
        std::vector<uint32_t> dp;
        for (uint32_t q : primes_upto(job->p))
            if (job->d % q == 0) dp.push_back(q);
        for (uint64_t mi = 0; mi < job->minc; mi++) {
            bool ok = true;
            for (uint32_t q : dp)
                if ((job->mstart + mi) % q == 0) {
                    ok = false;
                    break;
                }
            valid += ok;
        }
        out->valid_ms = valid;
    }
    return rc;
}

int pgs_prepare(pgs_ctx *ctx, const pgs_job *job, pgs_prepared **out) {
    if (!ctx || !job || !out) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    *out = nullptr;
    auto *pr = new pgs_prepared();
    pr->ctx = ctx;
    for (DevBuf *b : pr->all()) b->pool = &ctx->dpool;
    int rc = derive(*job, pr->hj, ctx->err, true);
    if (rc != PGS_OK) {
        delete pr;
        return rc;
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    HostJob &h = pr->hj;
    const uint64_t rows = h.valid_mi.size();

    // base primes for the whole sieve range (device; cached on the context)
    CK(pg::base_primes_build(ctx->base, h.prime_limit, s));

    // prime windows
    const uint32_t P = h.job.p;
    pr->sp_lo = (uint64_t)P + 1;
    pr->sp_hi = std::min<uint64_t>(h.s1, h.prime_limit);
    pr->sp_bound = pr->sp_hi >= pr->sp_lo ? pg::prime_count_bound(pr->sp_lo, pr->sp_hi) : 0;
    uint64_t lo = h.s1 + 1;
    while (lo <= h.prime_limit) {
        uint64_t hi = (lo / kWindowSpan + 1) * kWindowSpan - 1;
        if (hi > h.prime_limit) hi = h.prime_limit;
        Window w{lo, hi, pg::prime_count_bound(lo, hi), lo >= (1ull << 32)};
        pr->windows.push_back(w);
        pr->win_bound = std::max(pr->win_bound, w.bound);
        lo = hi + 1;
    }

    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    pr->events.push_back(e0);
    pr->events.push_back(e1);
    CK(cudaEventRecord(e0, s));
    // tables
    CK(upload(pr->klimbs, h.klimbs, s));
    CK(upload(pr->row_of_mi, h.row_of_mi, s));
    CK(upload(pr->col_of_x, h.col_of_x, s));
    CK(upload(pr->valid_mi, h.valid_mi, s));
    CK(upload(pr->dist, h.dist, s));
    CK(upload(pr->dq, h.dq, s));
    CK(upload(pr->mmask, h.mmask, s));
    CK(upload(pr->xmask, h.xmask, s));
    CK(pr->dr.ensure(std::max<size_t>(1, h.dq.size()) * 4));
    CK(cudaEventRecord(e1, s));
    // work buffers
    CK(pr->comp.ensure(rows * h.pitch * 4ull));
    CK(pr->sp.ensure(pr->sp_bound * 4 + 4));
    CK(pr->sr.ensure(pr->sp_bound * 4 + 4));
    CK(pr->sp_t0.ensure(pr->sp_bound * 4 + 4));
    CK(pr->lists.ensure(rows * 2ull * std::max<uint32_t>(h.H, 1) * 4));
    CK(pr->counts.ensure(rows * 2ull * 4));
    CK(pr->row_bytes.ensure(rows * 8ull));
    CK(pr->offsets.ensure(rows * 8ull));
    CK(pr->scan_tmp.ensure(pg::scan_tmp_words(rows) * 8));
    CK(pr->misc.ensure((2 + pr->windows.size()) * 8));
    {
        const uint64_t mmax = h.job.mstart + h.job.minc;
        uint64_t per_row = ndigits(mmax) + 2ull * ndigits(h.H) + 16;
        uint64_t per_entry = h.job.compression == 1 ? 2 : 2 + ndigits(h.job.sieve_length);
        pr->text_cap = rows * (per_row + 2ull * h.H * per_entry) + 64;
        CK(pr->text.ensure(pr->text_cap));
    }
    CK(ctx->win_off.ensure(pr->win_bound * 4 + 4));
    CK(ctx->win_r.ensure(pr->win_bound * 8 + 8));
    CK(ctx->win_t0.ensure(pr->win_bound * 8 + 8));
    CK(ctx->large_ctr.ensure(2 * sizeof(unsigned long long)));
    CK(ctx->heavy.ensure((size_t)pg::heavy_capacity() * pg::kHeavyPrimeBytes));
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    pr->ms_setup = ms;
    *out = pr;
    return PGS_OK;
}

int pgs_run(pgs_ctx *ctx, pgs_prepared *pr, int record_stages) {
    if (!ctx || !pr || pr->ctx != ctx) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    HostJob &h = pr->hj;
    const uint64_t rows = h.valid_mi.size();
    // the two setup events stay; stage events are rebuilt per run
    for (size_t i = 2; i < pr->events.size(); i++) cudaEventDestroy(pr->events[i]);
    pr->events.resize(2);
    pr->spans.clear();
    pr->launches = 0;
    auto mark = [&](int &idx) -> cudaError_t {
        idx = -1;
        if (!record_stages) return cudaSuccess;
        cudaEvent_t e;
        cudaError_t err = cudaEventCreate(&e);
        if (err) return err;
        pr->events.push_back(e);
        idx = (int)pr->events.size() - 1;
        return cudaEventRecord(e, s);
    };
    int a = -1, b = -1, first = -1;
    auto span = [&](int stage, int ea, int eb) {
        if (record_stages) pr->spans.push_back({stage, {ea, eb}});
    };

    const pg::JobDev job = job_dev(pr);
    const pg::RowsDev rd = rows_dev(pr);
    unsigned long long *misc = pr->misc.as<unsigned long long>();
    CK(mark(first));
    CK(cudaMemsetAsync(pr->comp.p, 0, rows * h.pitch * 4ull, s));
    CK(cudaMemsetAsync(pr->misc.p, 0, (2 + pr->windows.size()) * 8, s));

    // small primes (P, S1] and the odd primes of d
    if (pr->sp_bound) {
        CK(mark(a));
        CK(pg::sieve_window(ctx->base, pr->sp_lo, pr->sp_hi, pr->sp.as<uint32_t>(), pr->sp_bound,
                            misc + 1, s));
        CK(mark(b));
        span(PGS_STAGE_PRIMES, a, b);
        CK(pg::kmod_window(pr->klimbs.as<uint32_t>(), (int)h.klimbs.size(), pr->sp_lo,
                           pr->sp.as<uint32_t>(), misc + 1, pr->sp_bound, nullptr, pr->sr.p,
                           pr->sp_t0.p, false, s));
        CK(mark(a));
        span(PGS_STAGE_KMOD, b, a);
        pr->launches += 2;
    }
    if (!h.dq.empty()) {
        CK(pg::kmod_list32(pr->klimbs.as<uint32_t>(), (int)h.klimbs.size(), pr->dq.as<uint32_t>(),
                           (uint32_t)h.dq.size(), pr->dr.as<uint32_t>(), s));
        pr->launches += 1;
    }
    // large primes, window by window
    for (size_t w = 0; w < pr->windows.size(); w++) {
        const Window &win = pr->windows[w];
        unsigned long long *cnt = misc + 2 + w;
        int e_a, e_b, e_c, e_d;
        CK(mark(e_a));
        CK(pg::sieve_window(ctx->base, win.lo, win.hi, ctx->win_off.as<uint32_t>(), win.bound, cnt, s));
        CK(mark(e_b));
        CK(pg::kmod_window(pr->klimbs.as<uint32_t>(), (int)h.klimbs.size(), win.lo,
                           ctx->win_off.as<uint32_t>(), cnt, win.bound, &h.walk, ctx->win_r.p,
                           ctx->win_t0.p, win.wide, s));
        CK(mark(e_c));
        CK(pg::large_window(job, win.lo, ctx->win_off.as<uint32_t>(), cnt, win.bound, ctx->win_r.p,
                            ctx->win_t0.p, win.wide, pr->mmask.as<uint32_t>(),
                            pr->xmask.as<uint32_t>(),
                            pg::LargeScratch{ctx->large_ctr.as<unsigned long long>(),
                                             ctx->heavy.as<pg::HeavyPrime>(), pg::heavy_capacity()},
                            s));
        CK(mark(e_d));
        span(PGS_STAGE_PRIMES, e_a, e_b);
        span(PGS_STAGE_KMOD, e_b, e_c);
        span(PGS_STAGE_LARGE, e_c, e_d);
        pr->launches += 4;
    }
    // rows, text
    CK(mark(a));
    CK(pg::rows_extract(rd, rows_per_block(h.nb, h.job.compression), s));
    CK(mark(b));
    span(PGS_STAGE_ROWS, a, b);
    CK(pg::scan_u64(pr->row_bytes.as<uint64_t>(), pr->offsets.as<uint64_t>(), pr->misc.as<uint64_t>(),
                    rows, pr->scan_tmp.as<uint64_t>(), s));
    CK(pg::format_rows(rd, pr->offsets.as<uint64_t>(), pr->text.as<char>(), s));
    CK(mark(a));
    span(PGS_STAGE_TEXT, b, a);
    span(-1, first, a);
    pr->launches += 5;
    pr->ran = true;
    return PGS_OK;
}

int pgs_fetch(pgs_ctx *ctx, pgs_prepared *pr, pgs_result *out) {
    if (!ctx || !pr || !out || !pr->ran) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    memset(out, 0, sizeof(*out));
    HostJob &h = pr->hj;
    std::vector<uint64_t> misc(2 + pr->windows.size());
    CK(cudaMemcpyAsync(misc.data(), pr->misc.p, misc.size() * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint64_t total = misc[0];
    if (total > pr->text_cap) {
        ctx->err = "text larger than its bound";
        return PGS_ECUDA;
    }
    size_t cap = 0;
    char *host = pinned_pool().get(total + 1, &cap);
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
    float ms_d2h = 0;
    cudaEventElapsedTime(&ms_d2h, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);

    out->text = host;
    out->text_len = total;
    out->internal = new PinnedOwner{cap};
    out->rows = h.valid_mi.size();
    uint64_t primes = h.primes_to_P + misc[1];
    for (size_t w = 0; w < pr->windows.size(); w++) primes += misc[2 + w];
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

int pgs_stage_ms(pgs_ctx *ctx, pgs_prepared *pr, double *out, double *total) {
    if (!ctx || !pr || !out || !pr->ran) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < PGS_NSTAGES; i++) out[i] = 0;
    out[PGS_STAGE_SETUP] = pr->ms_setup;
    if (total) *total = 0;
    for (auto &sp : pr->spans) {
        if (sp.second.first < 0 || sp.second.second < 0) continue;
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, pr->events[sp.second.first], pr->events[sp.second.second]));
        if (sp.first < 0) {
            if (total) *total = ms;
        } else {
            out[sp.first] += ms;
        }
    }
    return PGS_OK;
}

int pgs_int_peak(pgs_ctx *ctx, double *imad_per_s) {
    if (!ctx || !imad_per_s) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    CK(pg::tools_imad_peak(imad_per_s, ctx->stream));
    return PGS_OK;
}

void pgs_prepared_free(pgs_prepared *pr) {
    if (!pr) return;
    if (pr->ctx) {
        cudaSetDevice(pr->ctx->device);
        cudaStreamSynchronize(pr->ctx->stream);
    }
    delete pr;
}

void pgs_result_free(pgs_result *r) {
    if (!r) return;
    if (r->text && r->internal) {
        auto *own = (PinnedOwner *)r->internal;
        pinned_pool().put(r->text, own->cap);
        delete own;
    }
    r->text = nullptr;
    r->internal = nullptr;
    r->text_len = 0;
}

int pgs_method2(pgs_ctx *ctx, const pgs_job *job, pgs_result *out) {
    if (!ctx || !job || !out) return PGS_EINVAL;
    pgs_prepared *pr = nullptr;
    int rc = pgs_prepare(ctx, job, &pr);
    if (rc) return rc;
    rc = pgs_run(ctx, pr, 1);
    if (rc == PGS_OK) rc = pgs_fetch(ctx, pr, out);
    pgs_prepared_free(pr);
    return rc;
}

int pgs_primes(pgs_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *out, size_t cap, size_t *count) {
    if (!ctx || !count || hi > 40000000000000ull) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    std::vector<uint64_t> all;
    if (lo <= 2 && hi >= 2) all.push_back(2);
    if (hi >= 3) {
        CK(pg::base_primes_build(ctx->base, hi, s));
        uint64_t a = std::max<uint64_t>(lo, 3);
        DevBuf buf, cnt;
        CK(cnt.ensure(8));
        while (a <= hi) {
            uint64_t b = std::min<uint64_t>(hi, (a / kWindowSpan + 1) * kWindowSpan - 1);
            uint64_t bound = pg::prime_count_bound(a, b);
            CK(buf.ensure(bound * 4 + 4));
            CK(cudaMemsetAsync(cnt.p, 0, 8, s));
            CK(pg::sieve_window(ctx->base, a, b, buf.as<uint32_t>(), bound, cnt.as<unsigned long long>(), s));
            uint64_t n = 0;
            CK(cudaMemcpyAsync(&n, cnt.p, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (n > bound) n = bound;
            std::vector<uint32_t> offs(n);
            if (n) CK(cudaMemcpy(offs.data(), buf.p, n * 4, cudaMemcpyDeviceToHost));
            for (uint32_t o : offs) all.push_back(a + o);
            a = b + 1;
        }
        buf.release();
        cnt.release();
    }
    std::sort(all.begin(), all.end());
    *count = all.size();
    if (out)
        for (size_t i = 0; i < all.size() && i < cap; i++) out[i] = all[i];
    return PGS_OK;
}

int pgs_k_mod_p(pgs_ctx *ctx, const uint32_t *k_limbs, int n_limbs, const uint64_t *q, size_t n,
                uint64_t *out) {
    if (!ctx || !k_limbs || n_limbs <= 0 || (!q && n)) return PGS_EINVAL;
    for (size_t i = 0; i < n; i++)
        if (q[i] < 3 || !(q[i] & 1) || q[i] >= (1ull << 46)) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevBuf dl, dq, dout;
    CK(dl.ensure(n_limbs * 4));
    CK(dq.ensure(n * 8 + 8));
    CK(dout.ensure(n * 8 + 8));
    CK(cudaMemcpyAsync(dl.p, k_limbs, n_limbs * 4, cudaMemcpyHostToDevice, s));
    if (n) CK(cudaMemcpyAsync(dq.p, q, n * 8, cudaMemcpyHostToDevice, s));
    CK(pg::tools_kmod_list64(dl.as<uint32_t>(), n_limbs, dq.as<uint64_t>(), n, dout.as<uint64_t>(), s));
    if (n) CK(cudaMemcpyAsync(out, dout.p, n * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    dl.release();
    dq.release();
    dout.release();
    return PGS_OK;
}

int pgs_modulo_search(pgs_ctx *ctx, const uint64_t *p, const uint64_t *a, const uint64_t *l,
                      const uint64_t *r, uint64_t *k_out, size_t n) {
    if (!ctx) return PGS_EINVAL;
    for (size_t i = 0; i < n; i++) {
        // 0 < a < p, 1 <= l <= r < p (modulo_search.h:20-31), p < 2^46
        if (p[i] >= (1ull << 46) || a[i] == 0 || a[i] >= p[i] || l[i] == 0 || l[i] > r[i] ||
            r[i] >= p[i])
            return PGS_EINVAL;
    }
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevBuf b;
    CK(b.ensure(5 * n * 8 + 8));
    uint64_t *d = b.as<uint64_t>();
    if (n) {
        CK(cudaMemcpyAsync(d, p, n * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d + n, a, n * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d + 2 * n, l, n * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d + 3 * n, r, n * 8, cudaMemcpyHostToDevice, s));
        CK(pg::tools_modsearch(d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, n, s));
        CK(cudaMemcpyAsync(k_out, d + 4 * n, n * 8, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    b.release();
    return PGS_OK;
}

int pgs_large_hits(pgs_ctx *ctx, uint64_t M, uint32_t max_mi, uint32_t SL, uint64_t prime,
                   uint64_t base_r, uint32_t *mi_out, uint64_t *mod_out, size_t cap,
                   size_t *count) {
    if (!ctx || !count) return PGS_EINVAL;
    if (prime <= 4ull * SL + 2 || prime >= (1ull << 46) || base_r == 0 || base_r >= prime)
        return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevBuf bmi, bmod, bcnt;
    CK(bmi.ensure(cap * 4 + 4));
    CK(bmod.ensure(cap * 8 + 8));
    CK(bcnt.ensure(8));
    CK(pg::tools_large_hits(M, max_mi, SL, prime, base_r, bmi.as<uint32_t>(), bmod.as<uint64_t>(),
                            cap, bcnt.as<unsigned long long>(), s));
    uint64_t n = 0;
    CK(cudaMemcpyAsync(&n, bcnt.p, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    size_t w = n < cap ? n : cap;
    if (w) {
        CK(cudaMemcpy(mi_out, bmi.p, w * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(mod_out, bmod.p, w * 8, cudaMemcpyDeviceToHost));
    }
    *count = n;
    bmi.release();
    bmod.release();
    bcnt.release();
    return PGS_OK;
}

}  // extern "C"
