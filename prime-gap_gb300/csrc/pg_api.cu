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

#include "pg_host.h"

using namespace pgh;

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
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) ctx->device_name = prop.name;
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
    ctx->win_off2.release();
    ctx->win_r2.release();
    ctx->win_t02.release();
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    ctx->large_ctr.release();
    ctx->heavy.release();
    ctx->walks.release();
    batch_state_destroy(ctx);
    ctx->dpool.trim();
    if (ctx->copy) cudaStreamDestroy(ctx->copy);
    for (cudaStream_t c : ctx->chunk)
        if (c) cudaStreamDestroy(c);
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
    pr->tune = tuning_for(ctx, *job);
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
    CK(upload_tables(pr, s));
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
    CK(pr->misc.ensure((3 + 2 * pr->windows.size() + kTextChunks) * 8));
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
    if (pr->windows.size() > 1) {
        CK(ctx->win_off2.ensure(pr->win_bound * 4 + 4));
        CK(ctx->win_r2.ensure(pr->win_bound * 8 + 8));
        CK(ctx->win_t02.ensure(pr->win_bound * 8 + 8));
    }
    CK(ctx->large_ctr.ensure(pg::kLargeCounters * sizeof(unsigned long long)));
    CK(ctx->heavy.ensure((size_t)pg::heavy_capacity() * pg::kHeavyPrimeBytes));
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    pr->ms_setup = ms;
    *out = pr;
    return PGS_OK;
}

namespace {

// The rows, their offsets and their text in kTextChunks chunks of rows, each
// chunk's text copied to pinned host memory on the context's copy stream as
// soon as it is written, while the next chunks' rows are sieved.  The chunk
// ends (running text offsets) are scanned on the device with a carry-in; the
// host reads each end from the chunk's event and sizes the host buffer from
// the first chunk (rows are alike), moving to an exact buffer in the rare
// case that a later chunk overruns the estimate.
int text_pipeline(pgs_ctx *ctx, pgs_prepared *pr, const pg::RowsDev &rd, uint32_t rpb, cudaStream_t s,
                  HostText &sink) {
    const uint32_t rows = (uint32_t)pr->hj.valid_mi.size();
    const uint32_t nblk = (rows + rpb - 1) / rpb;
    const uint32_t want = std::max<uint32_t>(1, std::min<uint32_t>(kTextChunks, pr->tune.text_chunks));
    const int C = (int)std::min<uint32_t>(want, std::max<uint32_t>(nblk, 1));
    std::vector<uint32_t> rb(C + 1);
    for (int c = 0; c <= C; c++)
        rb[c] = (uint32_t)std::min<uint64_t>(rows, (uint64_t)nblk * c / C * rpb);
    uint64_t *misc = pr->misc.as<uint64_t>();
    uint64_t *ends = misc + 3 + 2 * pr->windows.size();
    if (!ctx->copy) CK(cudaStreamCreateWithFlags(&ctx->copy, cudaStreamNonBlocking));
    if (!ctx->chunk[0]) {
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        for (int c = 0; c < kTextChunks; c++)
            CK(cudaStreamCreateWithPriority(&ctx->chunk[c], cudaStreamNonBlocking, std::min(least, greatest + c)));
    }
    cudaStream_t cs = ctx->copy;
    PinnedPool &pool = pinned_pool();
    size_t ecap = 0, cap = 0;
    uint64_t *h_ends = (uint64_t *)pool.get(kTextChunks * 8, &ecap);
    if (!h_ends) {
        ctx->err = "cudaMallocHost failed";
        return PGS_ENOMEM;
    }
    char *host = nullptr;
    // each chunk on its own stream: the rows kernels of all chunks run
    // together (earlier chunks' CTAs first), so no chunk ends in a partial
    // wave; the scans run in chunk order (each adds the previous chunk's end)
    std::vector<cudaEvent_t> ev(C, nullptr), scanned(C, nullptr);
    cudaEvent_t t0 = nullptr, t1 = nullptr, ready = nullptr;
    cudaError_t e = cudaSuccess;
    int rc = PGS_OK;
    for (int c = 0; c < C && e == cudaSuccess; c++) {
        e = cudaEventCreateWithFlags(&ev[c], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&scanned[c], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ready, s);
    for (int c = 0; c < C && e == cudaSuccess; c++) {
        cudaStream_t sc = ctx->chunk[c];
        e = cudaStreamWaitEvent(sc, ready, 0);
        if (e == cudaSuccess) e = pg::rows_extract(rd, rpb, sc, rb[c], rb[c + 1]);
        if (e == cudaSuccess && c) e = cudaStreamWaitEvent(sc, scanned[c - 1], 0);
        if (e == cudaSuccess)
            e = pg::scan_u64(pr->row_bytes.as<uint64_t>() + rb[c], pr->offsets.as<uint64_t>() + rb[c], ends + c,
                             rb[c + 1] - rb[c], pr->scan_tmp.as<uint64_t>(), sc, c ? ends + c - 1 : nullptr);
        if (e == cudaSuccess) e = cudaEventRecord(scanned[c], sc);
        if (e == cudaSuccess)
            e = pg::format_rows(rd, pr->offsets.as<uint64_t>(), pr->text.as<char>(), sc, rb[c], rb[c + 1]);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_ends + c, ends + c, 8, cudaMemcpyDeviceToHost, sc);
        if (e == cudaSuccess) e = cudaEventRecord(ev[c], sc);
        pr->launches += 5;
    }
    // the job's stream continues after every chunk
    for (int c = 0; c < C && e == cudaSuccess; c++) e = cudaStreamWaitEvent(s, ev[c], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(misc, ends + C - 1, 8, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(t0, cs);
    for (int c = 0; c < C && e == cudaSuccess && rc == PGS_OK; c++) {
        if ((e = cudaEventSynchronize(ev[c]))) break;
        const uint64_t lo = c ? h_ends[c - 1] : 0, hi = h_ends[c];
        if (hi > pr->text_cap) {
            ctx->err = "text larger than its bound";
            rc = PGS_ECUDA;
            break;
        }
        if (!host) {
            // text of the whole job, estimated from its first chunk (the
            // factor can be lowered through PGSIEVE_TEXT_ESTIMATE, which the
            // tests use to take the exact-buffer path)
            const char *fe = getenv("PGSIEVE_TEXT_ESTIMATE");
            const double f = fe ? atof(fe) : 1.1;
            uint64_t est = (uint64_t)((double)hi * rows / std::max<uint32_t>(rb[c + 1], 1) * f) +
                           (f >= 1.0 ? 65536 : 0);
            est = std::min<uint64_t>(std::max<uint64_t>(est, hi), pr->text_cap);
            if (!(host = pool.get(est + 1, &cap))) rc = PGS_ENOMEM;
        } else if (hi + 1 > cap) {
            // the estimate was short: wait for the whole text, then move the
            // part copied so far to a buffer of the exact size
            uint64_t total = 0;
            if ((e = cudaEventSynchronize(ev[C - 1])) || (e = cudaStreamSynchronize(cs))) break;
            total = h_ends[C - 1];
            size_t ncap = 0;
            char *nh = pool.get(total + 1, &ncap);
            if (!nh) {
                rc = PGS_ENOMEM;
                break;
            }
            memcpy(nh, host, lo);
            pool.put(host, cap);
            host = nh, cap = ncap;
        }
        if (rc == PGS_OK && hi > lo)
            e = cudaMemcpyAsync(host + lo, pr->text.as<char>() + lo, hi - lo, cudaMemcpyDeviceToHost, cs);
    }
    if (e == cudaSuccess && rc == PGS_OK) e = cudaEventRecord(t1, cs);
    if (e == cudaSuccess && rc == PGS_OK) e = cudaStreamSynchronize(cs);
    if (e == cudaSuccess && rc == PGS_OK) {
        sink.total = C ? h_ends[C - 1] : 0;
        host[sink.total] = 0;
        sink.text = host, sink.cap = cap;
        cudaEventElapsedTime(&sink.ms_d2h, t0, t1);
        host = nullptr;
    }
    // nothing of this job may still run once it returns (an error can leave
    // chunks queued that the job's stream does not wait for)
    for (int c = 0; c < C; c++) cudaStreamSynchronize(ctx->chunk[c]);
    cudaStreamSynchronize(cs);
    if (host) pool.put(host, cap);
    pool.put((char *)h_ends, ecap);
    for (int c = 0; c < C; c++) {
        if (ev[c]) cudaEventDestroy(ev[c]);
        if (scanned[c]) cudaEventDestroy(scanned[c]);
    }
    if (ready) cudaEventDestroy(ready);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (e != cudaSuccess) {
        ctx->err = cudaGetErrorString(e);
        return PGS_ECUDA;
    }
    if (rc == PGS_ENOMEM) ctx->err = "cudaMallocHost failed";
    return rc;
}

// One run of a prepared job (context locked).  With `sink`, the rows and
// text are pipelined with their copy to the host (text_pipeline).
int run_job_on(pgs_ctx *ctx, pgs_prepared *pr, int record_stages, HostText *sink, bool per_m) {
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    HostJob &h = pr->hj;
    const uint64_t rows = h.valid_mi.size();
    // the two setup events stay; stage events are rebuilt per run
    for (size_t i = 2; i < pr->events.size(); i++) cudaEventDestroy(pr->events[i]);
    pr->events.resize(2);
    pr->spans.clear();
    pr->launches = 0;
    auto mark_on = [&](int &idx, cudaStream_t st) -> cudaError_t {
        idx = -1;
        if (!record_stages) return cudaSuccess;
        cudaEvent_t e;
        cudaError_t err = cudaEventCreate(&e);
        if (err) return err;
        pr->events.push_back(e);
        idx = (int)pr->events.size() - 1;
        return cudaEventRecord(e, st);
    };
    auto mark = [&](int &idx) -> cudaError_t { return mark_on(idx, s); };
    int a = -1, b = -1, first = -1;
    auto span = [&](int stage, int ea, int eb) {
        if (record_stages) pr->spans.push_back({stage, {ea, eb}});
    };

    const pg::JobDev job = job_dev(pr);
    const pg::RowsDev rd = rows_dev(pr);
    unsigned long long *misc = pr->misc.as<unsigned long long>();
    CK(mark(first));
    CK(cudaMemsetAsync(pr->comp.p, 0, rows * h.pitch * 4ull, s));
    CK(cudaMemsetAsync(pr->misc.p, 0, (3 + 2 * pr->windows.size()) * 8, s));

    // The auxiliary stream: it makes what only the rows read, and later
    // windows' primes and K mod p, beside the job's stream, which it waits
    // on here and which waits on it before the rows.
    if (!ctx->aux) {
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CK(cudaStreamCreateWithPriority(&ctx->aux, cudaStreamNonBlocking, greatest));
    }
    cudaStream_t aux = ctx->aux;
    auto join = [&](cudaStream_t from, cudaStream_t to) -> cudaError_t {
        cudaEvent_t ev;
        cudaError_t err = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (err) return err;
        if ((err = cudaEventRecord(ev, from)) == cudaSuccess) err = cudaStreamWaitEvent(to, ev, 0);
        cudaEventDestroy(ev);
        return err;
    };
    CK(join(s, aux));

    // small primes (P, S1] and the odd primes of d, read by the rows only:
    // on the auxiliary stream, beside the first window's primes and K mod p
    if (pr->sp_bound) {
        CK(mark_on(a, aux));
        CK(pg::sieve_window(ctx->base, pr->sp_lo, pr->sp_hi, pr->sp.as<uint32_t>(), pr->sp_bound,
                            misc + 2, aux));
        CK(mark_on(b, aux));
        span(PGS_STAGE_PRIMES, a, b);
        CK(pg::kmod_window(pr->klimbs.as<uint32_t>(), (int)h.klimbs.size(), pr->sp_lo,
                           pr->sp.as<uint32_t>(), misc + 1, pr->sp_bound, nullptr, pr->sr.p,
                           nullptr, false, aux, 0, h.klimbs.data()));
        CK(mark_on(a, aux));
        span(PGS_STAGE_KMOD, b, a);
        pr->launches += 2;
    }
    if (!h.dq.empty()) {
        CK(pg::kmod_list32(pr->klimbs.as<uint32_t>(), (int)h.klimbs.size(), pr->dq.as<uint32_t>(),
                           (uint32_t)h.dq.size(), pr->dr.as<uint32_t>(), aux));
        pr->launches += 1;
    }
    // the warp-alone form's walk list, on first use
    if (pr->tune.large_form & 1u) CK(ctx->walks.ensure((size_t)pg::walk_capacity() * pg::kWalkEntryBytes));
    // K mod p of a window's primes inside the large-prime kernel: bit 1 of
    // the form for windows of 32-bit primes, bit 2 for 64-bit primes
    const bool limbs_fit = h.klimbs.size() <= (size_t)pg::kParamLimbs;
    // large primes, window by window, marking through the job descriptor jd.
    // With two or more windows the primes and K mod p of window w + 1 are
    // made on the auxiliary stream into the other buffer set while the large
    // primes of window w run on the job's stream: their CTAs take the SM
    // slots that the large-prime kernel's persistent CTAs give back as they
    // run out of groups, so the window's tail is not idle.  (Reserving slots
    // for them instead, two CTAs per SM, measured the same on the job of
    // P = 1511, SL = 2e4, 1e5 m, primes to 2e9, and cost the job of P = 3001,
    // SL = 4e4, 1e5 m, primes to 1e10 7.6 ms: its fused 64-bit kernel runs
    // only four CTAs per SM.)  The
    // stage times of the later windows' primes and K mod p are not recorded:
    // they run inside the large-prime spans.
    const size_t nwin = pr->windows.size();
    const bool overlap = nwin > 1;
    auto large_phase = [&](const pg::JobDev &jd) -> cudaError_t {
        if (nwin == 0) return cudaSuccess;  // every prime is a small one
        cudaError_t e;
        std::vector<cudaEvent_t> made(nwin, nullptr), used(nwin, nullptr);
        auto cleanup = [&]() {
            for (auto ev : made)
                if (ev) cudaEventDestroy(ev);
            for (auto ev : used)
                if (ev) cudaEventDestroy(ev);
        };
        // window w's primes and K mod p, on stream `ps`, into buffer set w & 1
        auto produce = [&](size_t w, cudaStream_t ps) -> cudaError_t {
            const Window &win = pr->windows[w];
            unsigned long long *rng = misc + 3 + 2 * w, *cnt = rng + 1;
            const bool second = overlap && (w & 1);
            uint32_t *off = second ? ctx->win_off2.as<uint32_t>() : ctx->win_off.as<uint32_t>();
            void *wr = second ? ctx->win_r2.p : ctx->win_r.p, *wt = second ? ctx->win_t02.p : ctx->win_t0.p;
            cudaError_t err;
            int e_a = -1, e_b = -1, e_c = -1;
            const bool timed = ps == s;  // the first window only
            if (timed && (err = mark_on(e_a, ps))) return err;
            if ((err = pg::sieve_window(ctx->base, win.lo, win.hi, off, win.bound, cnt, ps))) return err;
            if (timed && (err = mark_on(e_b, ps))) return err;
            const bool fuse = limbs_fit && (pr->tune.large_form & (win.wide ? 4u : 2u));
            if (!fuse &&
                (err = pg::kmod_window(pr->klimbs.as<uint32_t>(), (int)h.klimbs.size(), win.lo, off, rng, win.bound,
                                       &h.walk, wr, wt, win.wide, ps, (int)pr->tune.kmod_lsb_limbs,
                                       h.klimbs.data())))
                return err;
            if (timed) {
                if ((err = mark_on(e_c, ps))) return err;
                span(PGS_STAGE_PRIMES, e_a, e_b);
                span(PGS_STAGE_KMOD, e_b, e_c);
            }
            pr->launches += fuse ? 1 : 2;
            return cudaSuccess;
        };
        if ((e = produce(0, s))) return e;
        cudaEvent_t first_made = nullptr;
        if (overlap) {
            // the second window starts once the first one's K mod p is done,
            // so that it runs beside the first window's large primes
            if ((e = cudaEventCreateWithFlags(&first_made, cudaEventDisableTiming))) return e;
            if ((e = cudaEventRecord(first_made, s)) || (e = cudaStreamWaitEvent(ctx->aux, first_made, 0))) {
                cudaEventDestroy(first_made);
                return e;
            }
            cudaEventDestroy(first_made);
        }
        for (size_t w = 0; w < nwin; w++) {
            if (overlap && w + 1 < nwin) {
                // the next window on the auxiliary stream, once its buffers are free
                if (w >= 1 && (e = cudaStreamWaitEvent(ctx->aux, used[w - 1], 0))) break;
                if ((e = produce(w + 1, ctx->aux))) break;
                if ((e = cudaEventCreateWithFlags(&made[w + 1], cudaEventDisableTiming))) break;
                if ((e = cudaEventRecord(made[w + 1], ctx->aux))) break;
            }
            if (w >= 1 && overlap && (e = cudaStreamWaitEvent(s, made[w], 0))) break;
            const Window &win = pr->windows[w];
            unsigned long long *rng = misc + 3 + 2 * w;
            const bool second = overlap && (w & 1);
            const bool fuse = limbs_fit && (pr->tune.large_form & (win.wide ? 4u : 2u));
            int e_c, e_d;
            if ((e = mark(e_c))) break;
            e = pg::large_window(jd, win.lo, second ? ctx->win_off2.as<uint32_t>() : ctx->win_off.as<uint32_t>(), rng,
                                 win.bound, second ? ctx->win_r2.p : ctx->win_r.p,
                                 second ? ctx->win_t02.p : ctx->win_t0.p, rng, win.wide, false,
                                 pr->mmask.as<uint2>(), pr->ymask.as<uint2>(),
                                 pg::LargeScratch{ctx->large_ctr.as<unsigned long long>(),
                                                  ctx->heavy.as<pg::HeavyPrime>(), pg::heavy_capacity(),
                                                  ctx->walks.as<pg::WalkEntry>(),
                                                  ctx->walks.p ? pg::walk_capacity() : 0u},
                                 s, fuse ? h.klimbs.data() : nullptr, (int)h.klimbs.size(),
                                 pg::kmod_lsb((int)h.klimbs.size(), win.wide, (int)pr->tune.kmod_lsb_limbs));
            if (e) break;
            if ((e = mark(e_d))) break;
            span(PGS_STAGE_LARGE, e_c, e_d);
            if (overlap) {
                if ((e = cudaEventCreateWithFlags(&used[w], cudaEventDisableTiming))) break;
                if ((e = cudaEventRecord(used[w], s))) break;
            }
            // the large-prime kernel and the heavy list's, and the walks' in
            // the warp-alone form
            pr->launches += (pr->tune.large_form & 1u) && ctx->walks.p ? 3 : 2;
        }
        cleanup();
        return e;
    };
    if (!per_m) {
        CK(large_phase(job));
    } else {
        // The per-m path (method1, combined_sieve.cpp:409-751): the reference
        // keeps every large prime in a queue under the next m it divides and
        // sieves m by m.  Here the phase runs twice, first counting each
        // row's survivors, then, at offsets from their prefix sum, filing
        // each survivor's column under its row; each row's marks then come
        // from its own bucket.  Same bytes as method2.
        CK(pr->row_count.ensure(std::max<uint64_t>(rows, 1) * 8));
        CK(pr->row_off.ensure((rows + 1) * 8));
        unsigned long long *counts = pr->row_count.as<unsigned long long>();
        unsigned long long *offs = pr->row_off.as<unsigned long long>();  // rows + 1: the total last
        pg::JobDev jd = job;
        CK(cudaMemsetAsync(counts, 0, rows * 8, s));
        jd.mark_mode = pg::kMarkCount;
        jd.row_count = counts;
        CK(large_phase(jd));
        CK(pg::scan_u64((const uint64_t *)counts, (uint64_t *)offs, (uint64_t *)(offs + rows), rows,
                        pr->scan_tmp.as<uint64_t>(), s));
        uint64_t total = 0;
        CK(cudaMemcpyAsync(&total, offs + rows, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        CK(pr->bucket.ensure(std::max<uint64_t>(total, 1) * 4));
        CK(cudaMemsetAsync(counts, 0, rows * 8, s));  // now the fill position of each bucket
        // the windows' prime counts accumulate: start them again
        CK(cudaMemsetAsync(misc + 3, 0, 2 * pr->windows.size() * 8, s));
        jd.mark_mode = pg::kMarkBucket;
        jd.row_off = offs;
        jd.bucket = pr->bucket.as<uint32_t>();
        CK(large_phase(jd));
        CK(pg::bucket_apply(jd, offs + rows, s));
        pr->launches += 2;
    }
    // rows, text, once the auxiliary stream's small primes are made
    CK(join(aux, s));
    CK(mark(a));
    if (sink) {
        // rows and text interleave with the copy: one span for both
        const int rc = text_pipeline(ctx, pr, rd, rows_per_block(h.nb, h.job.compression, pr->tune.rows_per_cta), s, *sink);
        if (rc) return rc;
        CK(mark(b));
        span(PGS_STAGE_ROWS, a, b);
        span(-1, first, b);
        pr->ran = true;
        return PGS_OK;
    }
    CK(pg::rows_extract(rd, rows_per_block(h.nb, h.job.compression, pr->tune.rows_per_cta), s));
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

int run_job(pgs_ctx *ctx, pgs_prepared *pr, int record_stages, HostText *sink, bool per_m = false) {
    const int rc = run_job_on(ctx, pr, record_stages, sink, per_m);
    // nothing of a failed run may still be running on the auxiliary stream
    if (rc != PGS_OK && ctx->aux) cudaStreamSynchronize(ctx->aux);
    return rc;
}

}  // namespace

extern "C++" {
namespace pgh {
int run_prepared(pgs_ctx *ctx, pgs_prepared *pr, int record_stages, HostText *sink) {
    return run_job(ctx, pr, record_stages, sink);
}
}  // namespace pgh
}

int pgs_run(pgs_ctx *ctx, pgs_prepared *pr, int record_stages) {
    if (!ctx || !pr || pr->ctx != ctx) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    return run_job(ctx, pr, record_stages, nullptr);
}

int pgs_fetch(pgs_ctx *ctx, pgs_prepared *pr, pgs_result *out) {
    if (!ctx || !pr || !out || !pr->ran) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    return fetch_job(ctx, pr, ctx->stream, out);
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
    {
        // the text goes to the host chunk by chunk while later rows run
        std::lock_guard<std::mutex> g(ctx->mu);
        HostText ht;
        rc = run_job(ctx, pr, 1, &ht);
        if (rc == PGS_OK) {
            rc = fetch_job(ctx, pr, ctx->stream, out, &ht);
            if (rc != PGS_OK) pinned_pool().put(ht.text, ht.cap);
        }
    }
    pgs_prepared_free(pr);
    return rc;
}

int pgs_method1(pgs_ctx *ctx, const pgs_job *job, pgs_result *out) {
    if (!ctx || !job || !out) return PGS_EINVAL;
    pgs_prepared *pr = nullptr;
    int rc = pgs_prepare(ctx, job, &pr);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        HostText ht;
        rc = run_job(ctx, pr, 1, &ht, true);
        if (rc == PGS_OK) {
            rc = fetch_job(ctx, pr, ctx->stream, out, &ht);
            if (rc != PGS_OK) pinned_pool().put(ht.text, ht.cap);
        }
    }
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
