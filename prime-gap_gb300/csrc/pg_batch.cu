// Batched and served method2 over a prime table resident on the context.
//
// The plain path (pg_api.cu) sieves its own primes for every job.  Here all
// jobs share one table -- sorted primes in 2^30-wide windows plus the small
// primes of the row phase -- generated once and kept in HBM (every prime up to
// 4e9 is 760 MB as u32 offsets).  A job then costs K mod p, the large-prime
// walk and its rows only; it finds its primes by a device binary search
// (pg::find_range), so nothing waits on the host.
//
// Jobs run on lanes: CUDA streams with their own scratch (walk steps and
// starts, heavy-prime list).  A batch assigns its jobs to lanes by estimated
// cost (longest first onto the least-loaded lane) and is captured once as a
// CUDA graph spanning all lanes.  A server admits requests in arrival order
// as lanes free up and their device footprint fits a byte budget, and copies
// each result back as its lane's completion event fires.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <tuple>

#include "pg_host.h"

using namespace pgh;

struct TableWindow {
    uint64_t lo = 0, hi = 0, count = 0;
    DevBuf off;  // sorted primes as offsets from lo
};

struct PrimeTable {
    uint64_t small_limit = 0;  // sorted primes 3..small_limit in `small`
    DevBuf small;
    std::vector<uint32_t> small_host;
    std::vector<TableWindow *> windows;  // window k covers [max(3, k*2^30), (k+1)*2^30 - 1]
    uint64_t max_count = 0;
    ~PrimeTable() {
        for (auto *w : windows) {
            w->off.release();
            delete w;
        }
        small.release();
    }
};

struct Lane {
    cudaStream_t stream = nullptr;
    DevBuf r, t0, ctr, heavy;
    ~Lane() {
        r.release();
        t0.release();
        ctr.release();
        heavy.release();
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

constexpr uint64_t kSmallMin = 1ull << 22;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Extend the table to every prime <= limit and small primes <= small_need.
int table_extend(pgs_ctx *ctx, uint64_t limit, uint64_t small_need, cudaStream_t s) {
    if (!ctx->table) ctx->table = new PrimeTable();
    PrimeTable &t = *ctx->table;
    const uint64_t k_last = limit / kWindowSpan;
    const bool grow_small = small_need > t.small_limit;
    const uint64_t small_target = grow_small ? std::max(small_need, kSmallMin) : t.small_limit;
    if (!grow_small && t.windows.size() > k_last) return PGS_OK;
    const uint64_t cover = std::max((k_last + 1) * kWindowSpan - 1, small_target);
    CK(pg::base_primes_build(ctx->base, cover, s));
    struct Scratch {
        DevBuf tmp, cnt;
        ~Scratch() {
            tmp.release();
            cnt.release();
        }
    } sc;
    DevBuf &tmp = sc.tmp, &cnt = sc.cnt;
    tmp.pool = cnt.pool = &ctx->dpool;
    CK(cnt.ensure(8));
    if (grow_small) {
        // jobs in flight may read the old list: let them finish first
        for (Lane *l : ctx->lanes) CK(cudaStreamSynchronize(l->stream));
        const uint64_t cap = pg::prime_count_bound(0, small_target) + 16;
        CK(t.small.ensure(cap * 4));
        CK(tmp.ensure(pg::sieve_sorted_tmp_bytes(0, small_target)));
        CK(pg::sieve_window_sorted(ctx->base, 0, small_target, t.small.as<uint32_t>(), cap,
                                   cnt.as<unsigned long long>(), tmp.p, s));
        uint64_t n = 0;
        CK(cudaMemcpyAsync(&n, cnt.p, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        t.small_host.resize(n);
        if (n) CK(cudaMemcpy(t.small_host.data(), t.small.p, n * 4, cudaMemcpyDeviceToHost));
        t.small_limit = small_target;
    }
    for (uint64_t k = t.windows.size(); k <= k_last; k++) {
        auto *w = new TableWindow();
        w->lo = k == 0 ? 3 : k * kWindowSpan;
        w->hi = (k + 1) * kWindowSpan - 1;
        const uint64_t cap = pg::prime_count_bound(w->lo, w->hi) + 16;
        cudaError_t e = w->off.ensure(cap * 4);
        if (e == cudaSuccess) e = tmp.ensure(pg::sieve_sorted_tmp_bytes(w->lo, w->hi));
        if (e == cudaSuccess)
            e = pg::sieve_window_sorted(ctx->base, w->lo, w->hi, w->off.as<uint32_t>(), cap,
                                        cnt.as<unsigned long long>(), tmp.p, s);
        uint64_t n = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&n, cnt.p, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            w->off.release();
            delete w;
            return fail(ctx, e, "table window");
        }
        w->count = n;
        t.max_count = std::max(t.max_count, n);
        t.windows.push_back(w);
    }
    return PGS_OK;
}

// Size an idle lane's scratch for the largest table window.
int lane_buffers(pgs_ctx *ctx, Lane *l) {
    const uint64_t need = ctx->table ? ctx->table->max_count : 0;
    CK(l->r.ensure(need * 8 + 8));
    CK(l->t0.ensure(need * 8 + 8));
    CK(l->ctr.ensure(pg::kLargeCounters * sizeof(unsigned long long)));
    CK(l->heavy.ensure((size_t)pg::heavy_capacity() * pg::kHeavyPrimeBytes));
    return PGS_OK;
}

int ensure_lanes(pgs_ctx *ctx, int n) {
    while ((int)ctx->lanes.size() < n) {
        auto *l = new Lane();
        cudaError_t e = cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete l;
            return fail(ctx, e, "lane stream");
        }
        ctx->lanes.push_back(l);
    }
    for (int i = 0; i < n; i++) {
        int rc = lane_buffers(ctx, ctx->lanes[i]);
        if (rc) return rc;
    }
    return PGS_OK;
}

// Device bytes a job will hold (its tables and work buffers), from its
// derived parameters.
uint64_t job_footprint(const HostJob &h) {
    const uint64_t rows = h.valid_mi.size();
    const uint64_t mmax = h.job.mstart + h.job.minc;
    const uint64_t per_row = ndigits(mmax) + 2ull * ndigits(h.H) + 16;
    const uint64_t per_entry = h.job.compression == 1 ? 2 : 2 + ndigits(h.job.sieve_length);
    uint64_t b = rows * (per_row + 2ull * h.H * per_entry);     // text
    b += rows * h.pitch * 4ull + rows * 2ull * std::max<uint32_t>(h.H, 1) * 4;  // bitset, lists
    b += rows * (8 + 8 + 8 + 4);                                // counts, bytes, offsets, valid_mi
    b += (h.mmask.size() + h.ymask.size()) * 4ull;              // masks, rank counts
    return b;
}

// `derived`, when given, is the job's HostJob from derive(); it is moved in.
int prepare_table_job(pgs_ctx *ctx, const pgs_job &job, cudaStream_t s, pgs_prepared **out,
                      HostJob *derived = nullptr) {
    *out = nullptr;
    auto *pr = new pgs_prepared();
    pr->ctx = ctx;
    pr->table_mode = true;
    for (DevBuf *b : pr->all()) b->pool = &ctx->dpool;
    if (derived) {
        pr->hj = std::move(*derived);
    } else {
        int rc = derive(job, pr->hj, ctx->err, true);
        if (rc != PGS_OK) {
            delete pr;
            return rc;
        }
    }
    HostJob &h = pr->hj;
    // the tuner measures one-job runs; batched and served jobs keep the
    // defaults (per-class picks applied to the batch measured 1 % slower)
    pr->tune = pgt::tuning_default();
    PrimeTable &t = *ctx->table;
    const uint64_t rows = h.valid_mi.size();
    const uint64_t shi = std::min<uint64_t>(h.s1, h.prime_limit);
    if (shi > t.small_limit || h.prime_limit / kWindowSpan >= t.windows.size()) {
        ctx->err = "prime table does not cover the job";
        delete pr;
        return PGS_EINVAL;
    }
    // small primes (P, min(S1, limit)]: a contiguous run of the sorted table
    pr->tbl_a = std::upper_bound(t.small_host.begin(), t.small_host.end(), h.job.p) -
                t.small_host.begin();
    pr->tbl_b = std::upper_bound(t.small_host.begin(), t.small_host.end(), (uint32_t)shi) -
                t.small_host.begin();
    if (pr->tbl_b < pr->tbl_a) pr->tbl_b = pr->tbl_a;
    pr->sp_bound = pr->tbl_b - pr->tbl_a;
    for (size_t k = 0; k < t.windows.size(); k++)
        if (h.prime_limit > h.s1 && t.windows[k]->hi > h.s1 && t.windows[k]->lo <= h.prime_limit)
            pr->tbl_windows.push_back((int)k);

    cudaError_t e = cudaSuccess;
    e = upload_tables(pr, s);
    auto need = [&](DevBuf &b, size_t n) {
        if (e == cudaSuccess) e = b.ensure(n);
    };
    need(pr->dr, std::max<size_t>(1, h.dq.size()) * 4);
    need(pr->comp, rows * h.pitch * 4ull);
    need(pr->sr, pr->sp_bound * 4 + 4);
    need(pr->sp_t0, pr->sp_bound * 4 + 4);
    need(pr->lists, rows * 2ull * std::max<uint32_t>(h.H, 1) * 4);
    need(pr->counts, rows * 2ull * 4);
    need(pr->row_bytes, rows * 8ull);
    need(pr->offsets, rows * 8ull);
    need(pr->scan_tmp, pg::scan_tmp_words(rows) * 8);
    need(pr->misc, (1 + 2 * job_ranges(pr)) * 8);
    const uint64_t mmax = h.job.mstart + h.job.minc;
    const uint64_t per_row = ndigits(mmax) + 2ull * ndigits(h.H) + 16;
    const uint64_t per_entry = h.job.compression == 1 ? 2 : 2 + ndigits(h.job.sieve_length);
    pr->text_cap = rows * (per_row + 2ull * h.H * per_entry) + 64;
    need(pr->text, pr->text_cap);
    if (e != cudaSuccess) {
        delete pr;
        return fail(ctx, e, "prepare batched job");
    }
    size_t fp = 0;
    for (DevBuf *b : pr->all()) fp += b->n;
    pr->footprint = fp;
    *out = pr;
    return PGS_OK;
}

// K mod p already resident for every prime of some table windows (the
// request server's cache), indexed by table window: K mod p, R^2 mod p and the
// device range {0, count} of the whole window.
struct ResidueSource {
    std::vector<const void *> a, b;
    std::vector<const unsigned long long *> full;
};

// A group of jobs with the same P: their K = P#/d are all multiples of
// K' = P#/L, L = lcm of their d, so one K' mod p pass per prime window serves
// every job, each scaling it by L/d (two Montgomery products) as its walk
// starts.  A group of one job uses its own K and walk-start mode.
struct GroupPlan {
    std::vector<int> jobs;          // indices into the batch
    std::vector<uint32_t> klimbs;   // K' (groups of two or more)
    std::vector<uint32_t> kmul;     // L/d per job
    uint64_t cost = 0;
    int lane = 0;
};

// Kernels of one group on one lane, asynchronous and capturable: each job's
// setup (small primes, primes of d), then per table window one K' mod p pass
// over the hull of the jobs' prime ranges and every job's large-prime kernel
// reading from it, then each job's rows and text.  d_urange: 2 words per
// window of the hull; d_klimbs: K' on the device (both unused for one job).
int run_group(pgs_ctx *ctx, const std::vector<pgs_prepared *> &jobs, Lane *lane,
              unsigned long long *d_urange, const uint32_t *d_klimbs = nullptr, int nl_shared = 0,
              const std::vector<uint32_t> &kmul = {}, const ResidueSource *src = nullptr) {
    const cudaStream_t s = lane->stream;
    PrimeTable &t = *ctx->table;
    const pg::LargeScratch scratch{lane->ctr.as<unsigned long long>(), lane->heavy.as<pg::HeavyPrime>(),
                                   pg::heavy_capacity()};
    uint64_t lo_val = ~0ull, hi_val = 0;
    std::vector<int> windows;
    for (pgs_prepared *pr : jobs) {
        HostJob &h = pr->hj;
        const uint64_t rows = h.valid_mi.size();
        unsigned long long *misc = pr->misc.as<unsigned long long>();
        const int nl = (int)h.klimbs.size();
        pr->launches = 0;
        CK(cudaMemsetAsync(pr->comp.p, 0, rows * h.pitch * 4ull, s));
        CK(cudaMemsetAsync(pr->misc.p, 0, (1 + 2 * job_ranges(pr)) * 8, s));
        CK(pg::set_pair(misc + 1, pr->tbl_a, pr->tbl_b, s));
        pr->launches++;
        if (pr->sp_bound) {
            CK(pg::kmod_window(pr->klimbs.as<uint32_t>(), nl, 0, t.small.as<uint32_t>(), misc + 1,
                               pr->sp_bound, nullptr, pr->sr.p, nullptr, false, s));
            pr->launches++;
        }
        if (!h.dq.empty()) {
            CK(pg::kmod_list32(pr->klimbs.as<uint32_t>(), nl, pr->dq.as<uint32_t>(),
                               (uint32_t)h.dq.size(), pr->dr.as<uint32_t>(), s));
            pr->launches++;
        }
        if (!pr->tbl_windows.empty()) {
            lo_val = std::min(lo_val, h.s1 + 1);
            hi_val = std::max(hi_val, h.prime_limit);
        }
        windows.insert(windows.end(), pr->tbl_windows.begin(), pr->tbl_windows.end());
    }
    std::sort(windows.begin(), windows.end());
    windows.erase(std::unique(windows.begin(), windows.end()), windows.end());
    const bool shared = jobs.size() > 1;
    for (size_t u = 0; u < windows.size(); u++) {
        const TableWindow &w = *t.windows[windows[u]];
        const bool wide = w.lo >= (1ull << 32);
        // the jobs that sieve with this window, and their range slots
        std::vector<std::pair<pgs_prepared *, size_t>> users;
        std::vector<uint32_t> user_kmul;
        for (size_t j = 0; j < jobs.size(); j++)
            for (size_t i = 0; i < jobs[j]->tbl_windows.size(); i++)
                if (jobs[j]->tbl_windows[i] == windows[u]) {
                    users.push_back({jobs[j], i});
                    user_kmul.push_back(shared ? kmul[j] : 1u);
                }
        pgs_prepared *lead = users.front().first;
        if (src) {  // one job, K mod p resident for the whole window
            unsigned long long *rng = lead->misc.as<unsigned long long>() + 3 + 2 * users.front().second;
            CK(pg::find_range(w.off.as<uint32_t>(), w.count, w.lo, lead->hj.s1 + 1, lead->hj.prime_limit,
                              rng, s));
            const int k = windows[u];
            CK(pg::large_window(job_dev(lead), w.lo, w.off.as<uint32_t>(), rng, w.count, src->a[k], src->b[k],
                                src->full[k], wide, true, lead->mmask.as<uint2>(),
                                lead->ymask.as<uint2>(), scratch, s));
            lead->launches += 3;
            continue;
        }
        unsigned long long *rr;
        if (shared) {
            rr = d_urange + 2 * u;
            CK(pg::find_range(w.off.as<uint32_t>(), w.count, w.lo, lo_val, hi_val, rr, s));
        } else {
            rr = lead->misc.as<unsigned long long>() + 3 + 2 * users.front().second;
            CK(pg::find_range(w.off.as<uint32_t>(), w.count, w.lo, lead->hj.s1 + 1, lead->hj.prime_limit,
                              rr, s));
        }
        // one job: its walk step and start; a group: K' mod p, each job starts its own walk
        if (shared)
            CK(pg::kmod_window(d_klimbs, nl_shared, w.lo, w.off.as<uint32_t>(), rr, w.count, nullptr,
                               lane->r.p, lane->t0.p, wide, s));
        else
            CK(pg::kmod_window(lead->klimbs.as<uint32_t>(), (int)lead->hj.klimbs.size(), w.lo,
                               w.off.as<uint32_t>(), rr, w.count, &lead->hj.walk, lane->r.p,
                               lane->t0.p, wide, s));
        lead->launches += 2;
        for (size_t k = 0; k < users.size(); k++) {
            const auto &ui = users[k];
            pgs_prepared *pr = ui.first;
            pg::JobDev jd = job_dev(pr);
            jd.kmul = user_kmul[k];
            unsigned long long *rng = pr->misc.as<unsigned long long>() + 3 + 2 * ui.second;
            if (shared) {
                CK(pg::find_range(w.off.as<uint32_t>(), w.count, w.lo, pr->hj.s1 + 1, pr->hj.prime_limit,
                                  rng, s));
                pr->launches++;
            }
            CK(pg::large_window(jd, w.lo, w.off.as<uint32_t>(), rng, w.count, lane->r.p,
                                lane->t0.p, rr, wide, shared, pr->mmask.as<uint2>(),
                                pr->ymask.as<uint2>(), scratch, s));
            pr->launches += 2;
        }
    }
    for (pgs_prepared *pr : jobs) {
        HostJob &h = pr->hj;
        const uint64_t rows = h.valid_mi.size();
        pg::RowsDev rd = rows_dev(pr);
        rd.sp = t.small.as<uint32_t>();
        rd.sp_base = 0;
        rd.sp_range = pr->misc.as<unsigned long long>() + 1;
        rd.sp_cap = pr->sp_bound;
        CK(pg::rows_extract(rd, rows_per_block(h.nb, h.job.compression, pr->tune.rows_per_cta), s));
        CK(pg::scan_u64(pr->row_bytes.as<uint64_t>(), pr->offsets.as<uint64_t>(), pr->misc.as<uint64_t>(),
                        rows, pr->scan_tmp.as<uint64_t>(), s));
        CK(pg::format_rows(rd, pr->offsets.as<uint64_t>(), pr->text.as<char>(), s));
        pr->launches += 5;
        pr->ran = true;
    }
    return PGS_OK;
}

}  // namespace

namespace {

// derive() for many jobs on up to 8 host threads.  Returns the first failing
// job's status (and its message in err).
int derive_all(const pgs_job *jobs, int n, std::vector<HostJob> &out, bool tables, std::string &err) {
    out.assign(n, HostJob());
    std::vector<int> rc(n, PGS_OK);
    std::vector<std::string> msg(n);
    std::atomic<int> next{0};
    auto work = [&] {
        for (int i; (i = next.fetch_add(1)) < n;) rc[i] = derive(jobs[i], out[i], msg[i], tables);
    };
    const int T = std::max(1, std::min({8, n, (int)std::thread::hardware_concurrency()}));
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    for (int i = 0; i < n; i++)
        if (rc[i] != PGS_OK) {
            err = msg[i];
            return rc[i];
        }
    return PGS_OK;
}

// P#/L as 32-bit limbs, for L a product of distinct primes <= P.
std::vector<uint32_t> primorial_quotient(uint32_t P, uint64_t L) {
    std::vector<uint32_t> limbs{1};
    for (uint32_t q : primes_upto(P)) {
        if (L % q == 0) continue;
        uint64_t carry = 0;
        for (auto &l : limbs) {
            const uint64_t t = (uint64_t)l * q + carry;
            l = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) limbs.push_back((uint32_t)carry);
    }
    return limbs;
}

uint64_t gcd64(uint64_t a, uint64_t b) {
    while (b) {
        const uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace

// ---------------------------------------------------------------------------
// batch: every job's large-prime work in one tile-queue launch
//
// Jobs are grouped into chains: jobs whose P ascend P_1 < ... < P_G and whose
// d all divide one L (L | P_1#, every L/d below 2^32).  Per prime-table
// window one kmod_chain launch computes K'_g = P_g#/L mod p for every group
// of a chain in one pass over K'_G's limbs, and one large_multi launch then
// runs every job's primes of every window as tiles of 256 primes pulled from
// a device counter, each job starting its walks from its group's K' mod p
// scaled by L/d.  Ranges of every job in every window are found once at
// prepare time, so the launches have host-known tile counts and the whole
// batch is capturable as one CUDA graph.

namespace {

struct ChainPlan {
    std::vector<uint32_t> P;        // group primes, ascending
    uint64_t L = 1;
    std::vector<uint32_t> limbs;    // segments concatenated
    std::vector<uint32_t> seg_off;  // G + 1 limb offsets
    std::vector<int> jobs;
};

bool primes_of_L_below(uint64_t L, uint32_t P) {
    for (uint32_t q = 2; L > 1 && (uint64_t)q * q <= L; q++)
        while (L % q == 0) {
            if (q > P) return false;
            L /= q;
        }
    return L <= P;
}

// Chains over the distinct P ascending; a chain grows while the lcm of its d
// stays a divisor of P_1# with every L/d below 2^32 and its limbs fit the
// kernel's shared memory.
std::vector<ChainPlan> plan_chains(const std::vector<const HostJob *> &hj, std::vector<int> &chain_of,
                                   std::vector<int> &group_of, std::vector<uint32_t> &kmul) {
    std::map<uint32_t, std::vector<int>> by_p;
    for (int i = 0; i < (int)hj.size(); i++) by_p[hj[i]->job.p].push_back(i);
    std::vector<ChainPlan> out;
    chain_of.assign(hj.size(), -1);
    group_of.assign(hj.size(), 0);
    kmul.assign(hj.size(), 1);
    ChainPlan cur;
    auto fits = [&](const ChainPlan &c, uint64_t L, const std::vector<int> &more) {
        if (L == 0 || !primes_of_L_below(L, c.P.empty() ? hj[more[0]]->job.p : c.P.front())) return false;
        for (int i : c.jobs)
            if (L / hj[i]->job.d > 0xFFFFFFFFull) return false;
        for (int i : more)
            if (L / hj[i]->job.d > 0xFFFFFFFFull) return false;
        return true;
    };
    auto close = [&] {
        if (cur.jobs.empty()) return;
        // segment 0: P_1#/L; segment g: the primes in (P_(g-1), P_g]
        cur.limbs.clear();
        cur.seg_off.assign(1, 0);
        std::vector<uint32_t> seg = primorial_quotient(cur.P[0], cur.L);
        for (size_t g = 0; g < cur.P.size(); g++) {
            if (g) {
                seg.assign(1, 1);
                for (uint32_t q : primes_upto(cur.P[g])) {
                    if (q <= cur.P[g - 1]) continue;
                    uint64_t carry = 0;
                    for (auto &l : seg) {
                        const uint64_t t = (uint64_t)l * q + carry;
                        l = (uint32_t)t;
                        carry = t >> 32;
                    }
                    if (carry) seg.push_back((uint32_t)carry);
                }
            }
            cur.limbs.insert(cur.limbs.end(), seg.begin(), seg.end());
            cur.seg_off.push_back((uint32_t)cur.limbs.size());
        }
        const int c = (int)out.size();
        for (size_t g = 0; g < cur.P.size(); g++)
            for (int i : cur.jobs)
                if (hj[i]->job.p == cur.P[g]) chain_of[i] = c, group_of[i] = (int)g, kmul[i] = (uint32_t)(cur.L / hj[i]->job.d);
        out.push_back(std::move(cur));
        cur = ChainPlan();
    };
    for (auto &kv : by_p) {
        uint64_t L = cur.L;
        for (int i : kv.second) {
            const uint64_t d = hj[i]->job.d, g = gcd64(L, d);
            L = (L / g > (~0ull >> 1) / d) ? 0 : L / g * d;
            if (!L) break;
        }
        // the limbs of K'_G grow with P: keep well inside the kernel's shared memory
        const bool room = cur.limbs.size() + kv.first / 8 + 64 < 12000;
        if (!cur.jobs.empty() && !(room && fits(cur, L, kv.second))) {
            close();
            L = 1;
            for (int i : kv.second) {
                const uint64_t d = hj[i]->job.d, g = gcd64(L, d);
                L = (L / g > (~0ull >> 1) / d) ? 0 : L / g * d;
                if (!L) break;
            }
        }
        if (cur.jobs.empty() && !fits(cur, L, kv.second)) {
            // a P whose own d do not share one L: each d alone (L = d)
            for (int i : kv.second) {
                cur.P = {kv.first};
                cur.L = hj[i]->job.d;
                cur.jobs = {i};
                close();
            }
            continue;
        }
        cur.P.push_back(kv.first);
        cur.L = L;
        cur.jobs.insert(cur.jobs.end(), kv.second.begin(), kv.second.end());
    }
    close();
    return out;
}

}  // namespace

struct pgs_batch {
    pgs_ctx *ctx = nullptr;
    std::vector<pgs_prepared *> jobs;
    std::vector<int> lane_of;
    int nlanes = 1;
    // chains and their residues: per (chain, window) the union index range
    // of the chain's jobs in the window and G + 1 arrays of that length
    std::vector<ChainPlan> chains;
    std::vector<int> chain_of, group_of;
    std::vector<uint32_t> kmul;
    struct ChainWindow {
        int chain, window;
        uint64_t begin, count;
        bool wide;
        DevBuf r;  // G * count residues, then count R^2 values
    };
    std::vector<ChainWindow *> cw;
    DevBuf chain_limbs, chain_off;            // all chains' segments, offsets
    std::vector<size_t> limb_base, off_base;  // per chain
    // the tile launches in chunks of jobs: the rows of one chunk's jobs run
    // on the other lanes while the next chunk's large primes run
    struct Chunk {
        std::vector<int> jobs;
        DevBuf items32, items64;
        uint32_t n32 = 0, n64 = 0, tiles32 = 0, tiles64 = 0;
        cudaEvent_t done = nullptr;
    };
    std::vector<Chunk *> chunks;
    DevBuf d_jobs, counters, heavy;
    size_t smem = 0;
    bool all_shared = false;  // every job's masks fit shared memory
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr, fork = nullptr, setup_done = nullptr;
    std::vector<cudaEvent_t> joins, job_done;
    ~pgs_batch() {
        for (auto *c : cw) {
            c->r.release();
            delete c;
        }
        for (auto *c : chunks) {
            c->items32.release();
            c->items64.release();
            if (c->done) cudaEventDestroy(c->done);
            delete c;
        }
        for (DevBuf *d : {&chain_limbs, &chain_off, &d_jobs, &counters, &heavy}) d->release();
    }
};

namespace {

// Index ranges {begin, end} of [lo_val, hi_val] in table windows, found on
// the device and read back (prepare time).
int table_ranges(pgs_ctx *ctx, const std::vector<std::tuple<int, uint64_t, uint64_t>> &q,
                 std::vector<std::pair<uint64_t, uint64_t>> &out, cudaStream_t s) {
    out.assign(q.size(), {0, 0});
    if (q.empty()) return PGS_OK;
    DevBuf buf;
    buf.pool = &ctx->dpool;
    CK(buf.ensure(q.size() * 16));
    for (size_t i = 0; i < q.size(); i++) {
        const TableWindow &w = *ctx->table->windows[std::get<0>(q[i])];
        CK(pg::find_range(w.off.as<uint32_t>(), w.count, w.lo, std::get<1>(q[i]), std::get<2>(q[i]),
                          buf.as<unsigned long long>() + 2 * i, s));
    }
    std::vector<unsigned long long> h(2 * q.size());
    CK(cudaMemcpyAsync(h.data(), buf.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (size_t i = 0; i < q.size(); i++) out[i] = {h[2 * i], std::max(h[2 * i], h[2 * i + 1])};
    buf.release();
    return PGS_OK;
}

// Chains, residue buffers, jobs and tile items of a batch whose jobs are
// prepared (b->jobs) over the context's table.
int plan_batch(pgs_ctx *ctx, pgs_batch *b, cudaStream_t s) {
    PrimeTable &t = *ctx->table;
    const int n = (int)b->jobs.size();
    std::vector<const HostJob *> hp;
    for (auto *pr : b->jobs) hp.push_back(&pr->hj);
    b->chains = plan_chains(hp, b->chain_of, b->group_of, b->kmul);
    // chain x window union ranges, then every job's own range per window
    std::vector<std::tuple<int, uint64_t, uint64_t>> q;
    std::vector<std::pair<int, int>> qcw;
    for (int c = 0; c < (int)b->chains.size(); c++)
        for (int k = 0; k < (int)t.windows.size(); k++) {
            uint64_t lo = ~0ull, hi = 0;
            for (int j : b->chains[c].jobs)
                for (int w : b->jobs[j]->tbl_windows)
                    if (w == k) lo = std::min(lo, b->jobs[j]->hj.s1 + 1), hi = std::max(hi, b->jobs[j]->hj.prime_limit);
            if (lo <= hi) q.emplace_back(k, lo, hi), qcw.push_back({c, k});
        }
    const size_t nq_chain = q.size();
    std::vector<std::pair<int, int>> qjob;
    for (int j = 0; j < n; j++)
        for (int w : b->jobs[j]->tbl_windows) {
            q.emplace_back(w, b->jobs[j]->hj.s1 + 1, b->jobs[j]->hj.prime_limit);
            qjob.push_back({j, w});
        }
    std::vector<std::pair<uint64_t, uint64_t>> rg;
    int rc = table_ranges(ctx, q, rg, s);
    if (rc) return rc;
    std::map<std::pair<int, int>, pgs_batch::ChainWindow *> cw_of;
    for (size_t i = 0; i < nq_chain; i++) {
        auto *c = new pgs_batch::ChainWindow();
        c->chain = qcw[i].first;
        c->window = qcw[i].second;
        c->begin = rg[i].first;
        c->count = rg[i].second - rg[i].first;
        c->wide = t.windows[c->window]->lo >= (1ull << 32);
        c->r.pool = &ctx->dpool;
        b->cw.push_back(c);
        const size_t G = b->chains[c->chain].P.size();
        CK(c->r.ensure(std::max<uint64_t>(1, (G + 1) * c->count) * (c->wide ? 8 : 4)));
        cw_of[qcw[i]] = c;
    }
    // segments of every chain, packed
    std::vector<uint32_t> limbs, offs;
    for (const ChainPlan &c : b->chains) {
        b->limb_base.push_back(limbs.size());
        b->off_base.push_back(offs.size());
        limbs.insert(limbs.end(), c.limbs.begin(), c.limbs.end());
        offs.insert(offs.end(), c.seg_off.begin(), c.seg_off.end());
    }
    b->chain_limbs.pool = b->chain_off.pool = &ctx->dpool;
    CK(upload(b->chain_limbs, limbs, s));
    CK(upload(b->chain_off, offs, s));
    // jobs and items
    std::vector<pg::LargeJob> lj(n);
    size_t smem = 0;
    bool all_shared = true;
    for (int j = 0; j < n; j++) {
        pgs_prepared *pr = b->jobs[j];
        lj[j].job = job_dev(pr);
        lj[j].job.kmul = b->kmul[j];
        lj[j].mmask = pr->mmask.as<uint2>();
        lj[j].ymask = pr->ymask.as<uint2>();
        const size_t mb = 8ull * ((lj[j].job.walk.jmax + 31) / 32 + (lj[j].job.walk.w + 31) / 32);
        lj[j].masks_in_shared = mb <= 96 * 1024;
        if (lj[j].masks_in_shared) smem = std::max(smem, mb);
        all_shared = all_shared && lj[j].masks_in_shared;
    }
    b->smem = smem;
    b->all_shared = all_shared;
    // chunks: jobs by rows work, longest first, cut where the cumulative
    // large-prime work (primes to the limit) passes each quarter
    std::vector<int> order(n);
    for (int j = 0; j < n; j++) order[j] = j;
    auto rows_work = [&](int j) { return (double)b->jobs[j]->hj.valid_mi.size() * (b->jobs[j]->hj.H + 64); };
    auto large_work = [&](int j) {
        const double lim = (double)b->jobs[j]->hj.prime_limit;
        return lim / std::log(std::max(lim, 3.0));
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return rows_work(x) > rows_work(y); });
    double total = 0;
    for (int j = 0; j < n; j++) total += large_work(j);
    const int nchunks = std::max(1, std::min(4, n));
    double acc = 0;
    for (int j : order) {
        const int c = std::min(nchunks - 1, (int)(acc / total * nchunks));
        while ((int)b->chunks.size() <= c) b->chunks.push_back(new pgs_batch::Chunk());
        b->chunks[c]->jobs.push_back(j);
        acc += large_work(j);
    }
    std::map<int, std::vector<size_t>> q_of_job;
    for (size_t i = 0; i < qjob.size(); i++) q_of_job[qjob[i].first].push_back(i);
    for (int j = 0; j < n; j++) {  // the large primes each job sieves (its result's prime count)
        uint64_t c = 0;
        for (size_t i : q_of_job[j]) c += rg[nq_chain + i].second - rg[nq_chain + i].first;
        b->jobs[j]->large_primes = c;
    }
    for (pgs_batch::Chunk *ch : b->chunks) {
        std::vector<pg::LargeItem> it32, it64;
        for (int j : ch->jobs)
            for (size_t i : q_of_job[j]) {
                const int w = qjob[i].second;
                const auto r = rg[nq_chain + i];
                if (r.second <= r.first) continue;
                pgs_batch::ChainWindow *c = cw_of.at({b->chain_of[j], w});
                const TableWindow &tw = *t.windows[w];
                const size_t width = c->wide ? 8 : 4;
                const size_t G = b->chains[c->chain].P.size();
                pg::LargeItem it{};
                it.job = (uint32_t)j;
                it.count = (uint32_t)(r.second - r.first);
                it.base = tw.lo;
                it.off = tw.off.as<uint32_t>() + r.first;
                it.a = (const char *)c->r.p + ((uint64_t)b->group_of[j] * c->count + (r.first - c->begin)) * width;
                it.b = (const char *)c->r.p + ((uint64_t)G * c->count + (r.first - c->begin)) * width;
                uint32_t &tiles = c->wide ? ch->tiles64 : ch->tiles32;
                it.tile0 = tiles;
                tiles += (it.count + pg::kLargeTile - 1) / pg::kLargeTile;
                (c->wide ? it64 : it32).push_back(it);
            }
        ch->n32 = (uint32_t)it32.size();
        ch->n64 = (uint32_t)it64.size();
        ch->items32.pool = ch->items64.pool = &ctx->dpool;
        CK(upload(ch->items32, it32, s));
        CK(upload(ch->items64, it64, s));
        CK(cudaEventCreateWithFlags(&ch->done, cudaEventDisableTiming));
    }
    // each job's setup, rows and text on one lane: the lanes other than lane
    // 0 (which runs the chunks' large primes), in chunk order
    const int first_rows_lane = b->nlanes > 1 ? 1 : 0;
    int next_lane = 0;
    b->lane_of.assign(n, 0);
    for (pgs_batch::Chunk *ch : b->chunks)
        for (int j : ch->jobs) b->lane_of[j] = first_rows_lane + next_lane++ % (b->nlanes - first_rows_lane);
    for (DevBuf *d : {&b->d_jobs, &b->counters, &b->heavy}) d->pool = &ctx->dpool;
    CK(upload(b->d_jobs, lj, s));
    CK(b->counters.ensure(16));
    CK(b->heavy.ensure((size_t)pg::heavy_capacity() * pg::kHeavyPrimeBytes));
    CK(cudaStreamSynchronize(s));
    return PGS_OK;
}

// Per-job kernels before the large phase: the bitset and range words
// cleared, K mod p of the job's small primes and of the primes of d.
int job_setup(pgs_ctx *ctx, pgs_prepared *pr, cudaStream_t s) {
    PrimeTable &t = *ctx->table;
    HostJob &h = pr->hj;
    const uint64_t rows = h.valid_mi.size();
    unsigned long long *misc = pr->misc.as<unsigned long long>();
    const int nl = (int)h.klimbs.size();
    pr->launches = 0;
    CK(cudaMemsetAsync(pr->comp.p, 0, rows * h.pitch * 4ull, s));
    CK(cudaMemsetAsync(pr->misc.p, 0, (1 + 2 * job_ranges(pr)) * 8, s));
    CK(pg::set_pair(misc + 1, pr->tbl_a, pr->tbl_b, s));
    pr->launches++;
    if (pr->sp_bound) {
        CK(pg::kmod_window(pr->klimbs.as<uint32_t>(), nl, 0, t.small.as<uint32_t>(), misc + 1, pr->sp_bound, nullptr,
                           pr->sr.p, nullptr, false, s, 0, h.klimbs.data()));
        pr->launches++;
    }
    if (!h.dq.empty()) {
        CK(pg::kmod_list32(pr->klimbs.as<uint32_t>(), nl, pr->dq.as<uint32_t>(), (uint32_t)h.dq.size(),
                           pr->dr.as<uint32_t>(), s));
        pr->launches++;
    }
    return PGS_OK;
}

// Rows, offsets and text of one job.
int job_rows(pgs_ctx *ctx, pgs_prepared *pr, cudaStream_t s) {
    PrimeTable &t = *ctx->table;
    HostJob &h = pr->hj;
    const uint64_t rows = h.valid_mi.size();
    pg::RowsDev rd = rows_dev(pr);
    rd.sp = t.small.as<uint32_t>();
    rd.sp_base = 0;
    rd.sp_range = pr->misc.as<unsigned long long>() + 1;
    rd.sp_cap = pr->sp_bound;
    CK(pg::rows_extract(rd, rows_per_block(h.nb, h.job.compression, pr->tune.rows_per_cta), s));
    CK(pg::scan_u64(pr->row_bytes.as<uint64_t>(), pr->offsets.as<uint64_t>(), pr->misc.as<uint64_t>(), rows,
                    pr->scan_tmp.as<uint64_t>(), s));
    CK(pg::format_rows(rd, pr->offsets.as<uint64_t>(), pr->text.as<char>(), s));
    pr->launches += 5;
    pr->ran = true;
    return PGS_OK;
}

// The whole batch, asynchronous and capturable: job setups over the lanes;
// on lane 0 the chains' K' mod p and the two tile-queue launches (32-bit and
// 64-bit windows); then rows and text over the lanes, each job's done event
// recorded, all lanes joined back into lane 0.
int launch_batch(pgs_ctx *ctx, pgs_batch *b) {
    Lane *l0 = ctx->lanes[0];
    const cudaStream_t s0 = l0->stream;
    CK(cudaEventRecord(b->fork, s0));
    for (int l = 1; l < b->nlanes; l++) CK(cudaStreamWaitEvent(ctx->lanes[l]->stream, b->fork, 0));
    for (size_t j = 0; j < b->jobs.size(); j++) {
        int rc = job_setup(ctx, b->jobs[j], ctx->lanes[b->lane_of[j]]->stream);
        if (rc) return rc;
    }
    for (int l = 1; l < b->nlanes; l++) {
        CK(cudaEventRecord(b->joins[l], ctx->lanes[l]->stream));
        CK(cudaStreamWaitEvent(s0, b->joins[l], 0));
    }
    PrimeTable &t = *ctx->table;
    for (pgs_batch::ChainWindow *c : b->cw) {
        const ChainPlan &ch = b->chains[c->chain];
        const TableWindow &w = *t.windows[c->window];
        const size_t width = c->wide ? 8 : 4;
        CK(pg::kmod_chain(b->chain_limbs.as<uint32_t>() + b->limb_base[c->chain],
                          b->chain_off.as<uint32_t>() + b->off_base[c->chain], (int)ch.P.size(), (int)ch.limbs.size(),
                          w.lo, w.off.as<uint32_t>() + c->begin, c->count, c->r.p,
                          (char *)c->r.p + ch.P.size() * c->count * width, c->wide, s0, ch.limbs.data(),
                          ch.seg_off.data()));
    }
    const pg::LargeScratch scr{b->counters.as<unsigned long long>(), b->heavy.as<pg::HeavyPrime>(),
                               pg::heavy_capacity()};
    for (pgs_batch::Chunk *ch : b->chunks) {
        CK(pg::large_multi(b->d_jobs.as<pg::LargeJob>(), ch->items32.as<pg::LargeItem>(), ch->n32, ch->tiles32,
                           b->smem, false, scr, s0, b->all_shared));
        if (ch->tiles64)
            CK(pg::large_multi(b->d_jobs.as<pg::LargeJob>(), ch->items64.as<pg::LargeItem>(), ch->n64, ch->tiles64,
                               b->smem, true, scr, s0, b->all_shared));
        CK(cudaEventRecord(ch->done, s0));
        for (int j : ch->jobs) {
            const cudaStream_t s = ctx->lanes[b->lane_of[j]]->stream;
            CK(cudaStreamWaitEvent(s, ch->done, 0));
            int rc = job_rows(ctx, b->jobs[j], s);
            if (rc) return rc;
            b->jobs[j]->launches += 4;  // its share of the chain and tile launches
            CK(cudaEventRecord(b->job_done[j], s));
        }
    }
    for (int l = 1; l < b->nlanes; l++) {
        CK(cudaEventRecord(b->joins[l], ctx->lanes[l]->stream));
        CK(cudaStreamWaitEvent(s0, b->joins[l], 0));
    }
    return PGS_OK;
}

// Prepare a batch: derive (host threads), extend the table, prepare every
// job (uploads on the context stream), plan chains and tiles.
int batch_create(pgs_ctx *ctx, const pgs_job *jobs, int n, int lanes, pgs_batch **out) {
    *out = nullptr;
    std::vector<HostJob> hj;
    int rc = derive_all(jobs, n, hj, true, ctx->err);
    if (rc) return rc;
    uint64_t limit = 3, small = kSmallMin;
    for (const HostJob &h : hj) {
        limit = std::max(limit, h.prime_limit);
        small = std::max(small, std::min<uint64_t>(h.s1, h.prime_limit));
    }
    rc = table_extend(ctx, limit, small, ctx->stream);
    if (rc) return rc;
    const int L = std::max(1, std::min(lanes, n));
    rc = ensure_lanes(ctx, L);
    if (rc) return rc;
    auto *b = new pgs_batch();
    b->ctx = ctx;
    b->nlanes = L;
    b->lane_of.assign(n, 0);
    for (int i = 0; i < n; i++) {
        pgs_prepared *pr = nullptr;
        rc = prepare_table_job(ctx, jobs[i], ctx->stream, &pr, &hj[i]);
        if (rc) {
            pgs_batch_free(b);
            return rc;
        }
        b->jobs.push_back(pr);
    }
    rc = plan_batch(ctx, b, ctx->stream);
    if (rc) {
        pgs_batch_free(b);
        return rc;
    }
    cudaError_t e = cudaEventCreate(&b->t0);
    if (!e) e = cudaEventCreate(&b->t1);
    if (!e) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&b->setup_done, cudaEventDisableTiming);
    b->joins.assign(L, nullptr);
    b->job_done.assign(n, nullptr);
    for (int l = 1; l < L && !e; l++) e = cudaEventCreateWithFlags(&b->joins[l], cudaEventDisableTiming);
    for (int j = 0; j < n && !e; j++) e = cudaEventCreateWithFlags(&b->job_done[j], cudaEventDisableTiming);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
    if (e) {
        pgs_batch_free(b);
        return fail(ctx, e, "batch events");
    }
    *out = b;
    return PGS_OK;
}

}  // namespace

extern "C" {

int pgs_table_reserve(pgs_ctx *ctx, uint64_t limit) {
    if (!ctx || limit > 40000000000000ull) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    return table_extend(ctx, limit, kSmallMin, ctx->stream);
}

int pgs_batch_prepare(pgs_ctx *ctx, const pgs_job *jobs, int n, int lanes, pgs_batch **out) {
    if (!ctx || !jobs || n <= 0 || !out) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    return batch_create(ctx, jobs, n, lanes, out);
}

int pgs_batch_run(pgs_ctx *ctx, pgs_batch *b, int use_graph, double *ms) {
    if (!ctx || !b || b->ctx != ctx) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    Lane *l0 = ctx->lanes[0];
    if (use_graph && !b->exec) {
        CK(cudaStreamBeginCapture(l0->stream, cudaStreamCaptureModeRelaxed));
        int rc = launch_batch(ctx, b);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(l0->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CK(e);
        b->graph = graph;
        CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    CK(cudaEventRecord(b->t0, l0->stream));
    if (use_graph) {
        CK(cudaGraphLaunch(b->exec, l0->stream));
    } else {
        int rc = launch_batch(ctx, b);
        if (rc) return rc;
    }
    CK(cudaEventRecord(b->t1, l0->stream));
    CK(cudaEventSynchronize(b->t1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, b->t0, b->t1));
    if (ms) *ms = t;
    return PGS_OK;
}

int pgs_batch_fetch(pgs_ctx *ctx, pgs_batch *b, int i, pgs_result *out) {
    if (!ctx || !b || !out || i < 0 || i >= (int)b->jobs.size()) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    if (!b->jobs[i]->ran) return PGS_EINVAL;
    return fetch_job(ctx, b->jobs[i], ctx->lanes[b->lane_of[i]]->stream, out);
}

void pgs_batch_free(pgs_batch *b) {
    if (!b) return;
    if (b->ctx) {
        cudaSetDevice(b->ctx->device);
        for (Lane *l : b->ctx->lanes) cudaStreamSynchronize(l->stream);
    }
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : {b->t0, b->t1, b->fork, b->setup_done})
        if (e) cudaEventDestroy(e);
    for (auto e : b->joins)
        if (e) cudaEventDestroy(e);
    for (auto e : b->job_done)
        if (e) cudaEventDestroy(e);
    for (auto *pr : b->jobs) delete pr;
    delete b;
}

// One pass: the batch prepared and launched without a graph, and each job's
// text copied to the host on the context stream as soon as its rows and text
// are done on its lane (in launch order of completion events), while other
// lanes still run.
int pgs_method2_batch(pgs_ctx *ctx, const pgs_job *jobs, int n, pgs_result *outs) {
    if (!ctx || !jobs || n <= 0 || !outs) return PGS_EINVAL;
    for (int i = 0; i < n; i++) memset(&outs[i], 0, sizeof(pgs_result));
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    pgs_batch *b = nullptr;
    int rc = batch_create(ctx, jobs, n, 8, &b);
    if (rc) return rc;
    rc = launch_batch(ctx, b);
    // fetch in the order the jobs' lanes finish them: lane by lane, each
    // lane's jobs in launch order
    std::vector<std::vector<int>> per_lane(b->nlanes);
    for (int j = 0; j < n; j++) per_lane[b->lane_of[j]].push_back(j);
    std::vector<size_t> next(b->nlanes, 0);
    for (int done = 0; rc == PGS_OK && done < n;) {
        bool any = false;
        for (int l = 0; l < b->nlanes && rc == PGS_OK; l++) {
            if (next[l] >= per_lane[l].size()) continue;
            const int j = per_lane[l][next[l]];
            const cudaError_t q = cudaEventQuery(b->job_done[j]);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                rc = fail(ctx, q, "batch job event");
                break;
            }
            cudaError_t e = cudaStreamWaitEvent(ctx->stream, b->job_done[j], 0);
            if (e) {
                rc = fail(ctx, e, "batch fetch order");
                break;
            }
            rc = fetch_job(ctx, b->jobs[j], ctx->stream, &outs[j]);
            next[l]++;
            done++;
            any = true;
        }
        if (!any && rc == PGS_OK) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (rc != PGS_OK)
        for (int i = 0; i < n; i++) pgs_result_free(&outs[i]);
    pgs_batch_free(b);
    return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// server
//
// Two threads.  The dispatcher admits requests in arrival order: it derives
// the head job (once), waits until a lane is free and the job's footprint
// fits the budget, uploads its tables and launches its kernels on the lane,
// then records the lane's event.  The completer polls the lanes' events;
// when a job's kernels are done it frees the lane at once (the job's text
// lives in the job's own buffers, not in lane scratch) and copies the text
// back on its own stream, then releases the job's memory from the budget.

namespace {

// Served requests with the same (P, d) share K mod p: computed once per
// table window (for all its primes) on first use and kept, least recently
// used first out, within a byte budget.  R^2 mod p depends on p alone and is
// kept once per window.
struct KEntry {
    DevBuf limbs;
    int nl = 0;
    std::vector<DevBuf> r;          // per table window
    std::vector<cudaEvent_t> ready; // per table window, recorded after the fill
    size_t bytes = 0;
    uint64_t last = 0;
    int refs = 0;
};
struct WinShared {
    DevBuf r2, full;
    cudaEvent_t ready = nullptr;
};

}  // namespace

namespace {

struct Request {
    uint64_t ticket = 0;
    pgs_job job{};
    double t_submit = 0, latency_ms = 0;
    int status = 1;  // 1 pending/running, else a PGS_ status
    pgs_result res{};
    pgs_prepared *pr = nullptr;
    uint64_t footprint = 0;
    HostJob *hj = nullptr;  // derived once, at the head of the queue
    int derive_rc = 1;
    KEntry *kentry = nullptr;  // cache entry in use
    ~Request() { delete hj; }
};

}  // namespace

struct pgs_server {
    pgs_ctx *ctx = nullptr;
    uint64_t budget = 0;
    // K mod p cache (dispatcher thread; refs under mu)
    std::map<std::pair<uint32_t, uint32_t>, KEntry *> kcache;
    std::vector<WinShared> wins;
    uint64_t kcache_bytes = 0, kcache_budget = 0, kclock = 0, kfills = 0, khits = 0;
    int nlanes = 1;
    std::mutex mu;
    std::condition_variable cv_done;
    std::deque<Request *> pending;
    std::map<uint64_t, Request *> reqs;
    std::vector<Request *> lane_req;   // job whose kernels run on the lane
    std::vector<cudaEvent_t> lane_done;
    cudaStream_t fetch_stream = nullptr, fetch_stream2 = nullptr;  // one per copy-back thread
    std::deque<std::pair<Request *, int>> fetch_queue;                // finished, not yet copied
    std::condition_variable cv_fetch;
    bool poll_done = false;
    std::thread fetcher, fetcher2;
    cudaStream_t up_stream = nullptr;    // table uploads of the staged request
    cudaEvent_t staged_ready = nullptr;  // recorded after them
    uint64_t next_ticket = 1, in_use = 0, running = 0, fetching = 0;
    bool stopping = false, dispatcher_done = false;
    std::thread dispatcher, completer;
    std::string err;
    // statistics
    std::vector<double> latencies;
    uint64_t submitted = 0, completed = 0, failed = 0, peak_bytes = 0, max_inflight = 0;
    double t_first = -1, t_last = 0, prep_s = 0, fetch_s = 0;
    double derive_s = 0, upload_s = 0, launch_s = 0, pinned_s0 = 0, dev_s0 = 0;
    uint64_t pinned_n0 = 0, dev_n0 = 0;
};

namespace {

// The (P, d) entry of the K mod p cache, created on first use.
KEntry *kcache_get(pgs_server *srv, const HostJob &h, cudaStream_t s, cudaError_t &e) {
    const auto key = std::make_pair(h.job.p, h.job.d);
    auto it = srv->kcache.find(key);
    if (it != srv->kcache.end()) return it->second;
    auto *ke = new KEntry();
    ke->limbs.pool = &srv->ctx->dpool;
    ke->nl = (int)h.klimbs.size();
    e = upload(ke->limbs, h.klimbs, s);
    if (e != cudaSuccess) {
        ke->limbs.release();
        delete ke;
        return nullptr;
    }
    srv->kcache[key] = ke;
    return ke;
}

void kentry_free(KEntry *ke) {
    for (auto &b : ke->r) b.release();
    for (auto ev : ke->ready)
        if (ev) cudaEventDestroy(ev);
    ke->limbs.release();
    delete ke;
}

// Make K mod p of every window the job uses resident (filling missing
// windows on stream s) and order s after the fills; fills src.
int kcache_prepare(pgs_server *srv, KEntry *ke, const pgs_prepared *pr, cudaStream_t s, ResidueSource &src) {
    pgs_ctx *ctx = srv->ctx;
    PrimeTable &t = *ctx->table;
    const size_t nw = t.windows.size();
    if (srv->wins.size() < nw) srv->wins.resize(nw);
    if (ke->r.size() < nw) {
        ke->r.resize(nw);
        ke->ready.resize(nw, nullptr);
    }
    src.a.assign(nw, nullptr);
    src.b.assign(nw, nullptr);
    src.full.assign(nw, nullptr);
    for (int k : pr->tbl_windows) {
        const TableWindow &w = *t.windows[k];
        const bool wide = w.lo >= (1ull << 32);
        const size_t width = wide ? 8 : 4;
        WinShared &ws = srv->wins[k];
        bool fill_r2 = false;
        if (!ws.full.p) {
            const std::vector<unsigned long long> full{0ull, (unsigned long long)w.count};
            CK(upload(ws.full, full, s));
            CK(ws.r2.ensure(w.count * width + 8));
            CK(cudaEventCreateWithFlags(&ws.ready, cudaEventDisableTiming));
            fill_r2 = true;
        }
        if (!ke->r[k].p) {
            ke->r[k].pool = &ctx->dpool;
            CK(ke->r[k].ensure(w.count * width + 8));
            CK(pg::kmod_window(ke->limbs.as<uint32_t>(), ke->nl, w.lo, w.off.as<uint32_t>(),
                               ws.full.as<unsigned long long>(), w.count, nullptr, ke->r[k].p,
                               fill_r2 ? ws.r2.p : nullptr, wide, s));
            CK(cudaEventCreateWithFlags(&ke->ready[k], cudaEventDisableTiming));
            CK(cudaEventRecord(ke->ready[k], s));
            if (fill_r2) CK(cudaEventRecord(ws.ready, s));
            ke->bytes += ke->r[k].n;
            srv->kcache_bytes += ke->r[k].n;
            srv->kfills++;
        } else {
            CK(cudaStreamWaitEvent(s, ke->ready[k], 0));
            srv->khits++;
        }
        CK(cudaStreamWaitEvent(s, ws.ready, 0));
        src.a[k] = ke->r[k].p;
        src.b[k] = ws.r2.p;
        src.full[k] = ws.full.as<unsigned long long>();
    }
    return PGS_OK;
}

// Drop least recently used entries no running job holds while over budget.
void kcache_trim(pgs_server *srv) {
    while (srv->kcache_bytes > srv->kcache_budget) {
        auto victim = srv->kcache.end();
        {
            std::lock_guard<std::mutex> g(srv->mu);
            for (auto it = srv->kcache.begin(); it != srv->kcache.end(); ++it)
                if (it->second->refs == 0 && (victim == srv->kcache.end() || it->second->last < victim->second->last))
                    victim = it;
        }
        if (victim == srv->kcache.end()) return;
        srv->kcache_bytes -= victim->second->bytes;
        kentry_free(victim->second);
        srv->kcache.erase(victim);
    }
}

void complete(pgs_server *srv, Request *r, int status, cudaStream_t fs) {
    const double t0 = now_s();
    if (status == PGS_OK) status = fetch_job(srv->ctx, r->pr, fs, &r->res);
    delete r->pr;
    r->pr = nullptr;
    const double t = now_s();
    std::lock_guard<std::mutex> g(srv->mu);
    srv->fetch_s += t - t0;
    r->latency_ms = (t - r->t_submit) * 1e3;
    r->status = status;
    srv->in_use -= r->footprint;
    srv->fetching--;
    if (r->kentry) r->kentry->refs--;
    r->kentry = nullptr;
    srv->t_last = t;
    if (status == PGS_OK) {
        srv->completed++;
        srv->latencies.push_back(r->latency_ms);
    } else {
        srv->failed++;
    }
    srv->cv_done.notify_all();
}

void complete_loop(pgs_server *srv) {
    cudaSetDevice(srv->ctx->device);
    for (;;) {
        bool idle = true;
        for (int l = 0; l < srv->nlanes; l++) {
            Request *r;
            {
                std::lock_guard<std::mutex> g(srv->mu);
                r = srv->lane_req[l];
            }
            if (!r) continue;
            cudaError_t q = cudaEventQuery(srv->lane_done[l]);
            if (q == cudaErrorNotReady) continue;
            {
                std::lock_guard<std::mutex> g(srv->mu);
                srv->lane_req[l] = nullptr;  // the lane takes new work now
                srv->running--;
                srv->fetching++;
                srv->fetch_queue.push_back({r, q == cudaSuccess ? PGS_OK : PGS_ECUDA});
            }
            srv->cv_fetch.notify_one();
            idle = false;
        }
        {
            std::lock_guard<std::mutex> g(srv->mu);
            if (srv->dispatcher_done && srv->running == 0) {
                srv->poll_done = true;
                srv->cv_fetch.notify_all();
                return;
            }
        }
        if (idle) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

// Copy-back threads: finished jobs' texts to the host, each on its own
// stream, so a slow copy (or a pinned allocation) never holds up the lane
// polling above.
void fetch_loop(pgs_server *srv, cudaStream_t fs) {
    cudaSetDevice(srv->ctx->device);
    for (;;) {
        std::pair<Request *, int> job;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            srv->cv_fetch.wait(lk, [&] { return !srv->fetch_queue.empty() || srv->poll_done; });
            if (srv->fetch_queue.empty()) return;
            job = srv->fetch_queue.front();
            srv->fetch_queue.pop_front();
        }
        complete(srv, job.first, job.second, fs);
    }
}

// A request that failed before or at launch leaves with its status.
void reject(pgs_server *srv, Request *r, int rc) {
    std::lock_guard<std::mutex> g(srv->mu);
    if (r->kentry) r->kentry->refs--;
    r->kentry = nullptr;
    delete r->pr;
    r->pr = nullptr;
    r->status = rc;
    srv->failed++;
    srv->cv_done.notify_all();
}

// Launch a staged request (tables uploaded on the upload stream) on a free lane.
int launch_staged(pgs_server *srv, Request *r, int lane) {
    pgs_ctx *ctx = srv->ctx;
    Lane *L = ctx->lanes[lane];
    int rc = lane_buffers(ctx, L);
    if (rc) return rc;
    cudaError_t ce = cudaSuccess;
    KEntry *ke = kcache_get(srv, r->pr->hj, L->stream, ce);
    if (!ke) return fail(ctx, ce, "K mod p cache");
    {
        std::lock_guard<std::mutex> g(srv->mu);
        ke->refs++;
        ke->last = ++srv->kclock;
        r->kentry = ke;
    }
    ResidueSource src;
    rc = kcache_prepare(srv, ke, r->pr, L->stream, src);
    if (rc) return rc;
    CK(cudaStreamWaitEvent(L->stream, srv->staged_ready, 0));
    rc = run_group(ctx, {r->pr}, L, nullptr, nullptr, 0, {}, &src);
    if (rc) return rc;
    CK(cudaEventRecord(srv->lane_done[lane], L->stream));
    return PGS_OK;
}

// Arrival order.  The head request is staged -- derived, admitted against
// the budget, its tables uploaded on the upload stream -- while the lanes are
// busy, and launched on the first lane that frees up.
void dispatch_loop(pgs_server *srv) {
    pgs_ctx *ctx = srv->ctx;
    cudaSetDevice(ctx->device);
    Request *staged = nullptr;
    for (;;) {
        bool progress = false;
        if (staged) {
            int lane = -1;
            {
                std::lock_guard<std::mutex> g(srv->mu);
                for (int l = 0; l < srv->nlanes && lane < 0; l++)
                    if (!srv->lane_req[l]) lane = l;
            }
            if (lane >= 0) {
                const double t0 = now_s();
                Request *r = staged;
                staged = nullptr;
                const int rc = launch_staged(srv, r, lane);
                kcache_trim(srv);
                if (rc != PGS_OK) {
                    {
                        std::lock_guard<std::mutex> g(srv->mu);
                        srv->in_use -= r->footprint;
                    }
                    reject(srv, r, rc);
                } else {
                    std::lock_guard<std::mutex> g(srv->mu);
                    srv->prep_s += now_s() - t0;
                    srv->launch_s += now_s() - t0;
                    srv->lane_req[lane] = r;
                    srv->running++;
                    srv->max_inflight = std::max(srv->max_inflight, srv->running + srv->fetching);
                    if (srv->t_first < 0) srv->t_first = now_s();
                }
                progress = true;
            }
        }
        if (!staged) {
            Request *r = nullptr;
            {
                std::lock_guard<std::mutex> g(srv->mu);
                if (!srv->pending.empty()) {
                    r = srv->pending.front();
                } else if (srv->stopping) {
                    srv->dispatcher_done = true;
                    return;
                }
            }
            if (r) {
                const double t0 = now_s();
                if (r->derive_rc == 1) {
                    r->hj = new HostJob();
                    r->derive_rc = derive(r->job, *r->hj, srv->err, true);
                    r->footprint = r->derive_rc == PGS_OK ? job_footprint(*r->hj) : 0;
                    std::lock_guard<std::mutex> g(srv->mu);
                    srv->derive_s += now_s() - t0;
                }
                const double t1 = now_s();
                int rc = r->derive_rc;
                bool admit = true;
                if (rc == PGS_OK) {
                    std::lock_guard<std::mutex> g(srv->mu);
                    // the head waits while it does not fit (unless nothing holds memory)
                    admit = srv->in_use == 0 || srv->in_use + r->footprint <= srv->budget;
                    if (admit) {
                        srv->in_use += r->footprint;
                        srv->peak_bytes = std::max(srv->peak_bytes, srv->in_use);
                    }
                }
                if (admit) {
                    {
                        std::lock_guard<std::mutex> g(srv->mu);
                        srv->pending.pop_front();
                    }
                    if (rc == PGS_OK) {
                        HostJob &h = *r->hj;
                        rc = table_extend(ctx, h.prime_limit, std::min<uint64_t>(h.s1, h.prime_limit),
                                          srv->up_stream);
                        if (rc == PGS_OK) rc = prepare_table_job(ctx, r->job, srv->up_stream, &r->pr, r->hj);
                        if (rc == PGS_OK && cudaEventRecord(srv->staged_ready, srv->up_stream) != cudaSuccess)
                            rc = PGS_ECUDA;
                    }
                    if (rc == PGS_OK) {
                        staged = r;
                        std::lock_guard<std::mutex> g(srv->mu);
                        srv->prep_s += now_s() - t0;
                        srv->upload_s += now_s() - t1;
                    } else {
                        if (r->derive_rc == PGS_OK) {
                            std::lock_guard<std::mutex> g(srv->mu);
                            srv->in_use -= r->footprint;
                        }
                        reject(srv, r, rc);
                    }
                    progress = true;
                }
            }
        }
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

}  // namespace

extern "C" {

int pgs_server_start(pgs_ctx *ctx, uint64_t hbm_budget, int lanes, pgs_server **out) {
    if (!ctx || !out || lanes <= 0) return PGS_EINVAL;
    *out = nullptr;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        int rc = table_extend(ctx, 3, kSmallMin, ctx->stream);
        if (rc) return rc;
        rc = ensure_lanes(ctx, lanes);
        if (rc) return rc;
    }
    auto *srv = new pgs_server();
    srv->ctx = ctx;
    srv->budget = hbm_budget;
    srv->kcache_budget = hbm_budget / 4;
    {
        PinnedPool &pp = pinned_pool();
        std::lock_guard<std::mutex> pg(pp.mu);
        srv->pinned_s0 = pp.alloc_s;
        srv->pinned_n0 = pp.allocs;
    }
    {
        DevicePool &dp = ctx->dpool;
        std::lock_guard<std::mutex> dg(dp.mu);
        srv->dev_s0 = dp.alloc_s;
        srv->dev_n0 = dp.allocs;
    }
    srv->nlanes = lanes;
    srv->lane_req.assign(lanes, nullptr);
    srv->lane_done.assign(lanes, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&srv->fetch_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&srv->fetch_stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&srv->up_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&srv->staged_ready, cudaEventDisableTiming);
    for (int l = 0; l < lanes && e == cudaSuccess; l++)
        e = cudaEventCreateWithFlags(&srv->lane_done[l], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        for (auto ev : srv->lane_done)
            if (ev) cudaEventDestroy(ev);
        if (srv->fetch_stream) cudaStreamDestroy(srv->fetch_stream);
        if (srv->fetch_stream2) cudaStreamDestroy(srv->fetch_stream2);
        if (srv->up_stream) cudaStreamDestroy(srv->up_stream);
        if (srv->staged_ready) cudaEventDestroy(srv->staged_ready);
        delete srv;
        return fail(ctx, e, "server start");
    }
    srv->dispatcher = std::thread(dispatch_loop, srv);
    srv->completer = std::thread(complete_loop, srv);
    srv->fetcher = std::thread(fetch_loop, srv, srv->fetch_stream);
    srv->fetcher2 = std::thread(fetch_loop, srv, srv->fetch_stream2);
    *out = srv;
    return PGS_OK;
}

int pgs_server_submit(pgs_server *srv, const pgs_job *job, uint64_t *ticket) {
    if (!srv || !job) return PGS_EINVAL;
    auto *r = new Request();
    r->job = *job;
    r->t_submit = now_s();
    std::lock_guard<std::mutex> g(srv->mu);
    if (srv->stopping) {
        delete r;
        return PGS_EINVAL;
    }
    r->ticket = srv->next_ticket++;
    srv->reqs[r->ticket] = r;
    srv->pending.push_back(r);
    srv->submitted++;
    if (ticket) *ticket = r->ticket;
    return PGS_OK;
}

int pgs_server_wait(pgs_server *srv, uint64_t ticket, int timeout_ms, pgs_result *out,
                    double *latency_ms) {
    if (!srv || !out) return PGS_EINVAL;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return PGS_EINVAL;
    Request *r = it->second;
    auto done = [&] { return r->status != 1; };
    if (timeout_ms < 0) {
        srv->cv_done.wait(lk, done);
    } else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
        return PGS_ETIMEOUT;
    }
    const int status = r->status;
    *out = r->res;
    if (latency_ms) *latency_ms = r->latency_ms;
    srv->reqs.erase(it);
    delete r;
    return status;
}

int pgs_server_stats_get(pgs_server *srv, pgs_server_stats *out) {
    if (!srv || !out) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(srv->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = srv->submitted;
    out->completed = srv->completed;
    out->failed = srv->failed;
    out->peak_bytes = srv->peak_bytes;
    out->max_inflight = srv->max_inflight;
    out->host_prep_s = srv->prep_s;
    out->host_fetch_s = srv->fetch_s;
    out->kmod_fills = srv->kfills;
    out->kmod_hits = srv->khits;
    out->host_derive_s = srv->derive_s;
    out->host_upload_s = srv->upload_s;
    out->host_launch_s = srv->launch_s;
    {
        PinnedPool &pp = pinned_pool();
        std::lock_guard<std::mutex> pg(pp.mu);
        out->pinned_alloc_s = pp.alloc_s - srv->pinned_s0;
        out->pinned_allocs = pp.allocs - srv->pinned_n0;
    }
    {
        DevicePool &dp = srv->ctx->dpool;
        std::lock_guard<std::mutex> dg(dp.mu);
        out->device_alloc_s = dp.alloc_s - srv->dev_s0;
        out->device_allocs = dp.allocs - srv->dev_n0;
    }
    if (!srv->latencies.empty()) {
        std::vector<double> v = srv->latencies;
        std::sort(v.begin(), v.end());
        auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
        out->max_ms = v.back();
        double s = 0;
        for (double x : v) s += x;
        out->mean_ms = s / v.size();
    }
    out->busy_s = srv->t_first >= 0 ? srv->t_last - srv->t_first : 0;
    return PGS_OK;
}

int pgs_server_stop(pgs_server *srv) {
    if (!srv) return PGS_EINVAL;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->stopping = true;
    }
    if (srv->dispatcher.joinable()) srv->dispatcher.join();
    if (srv->completer.joinable()) srv->completer.join();
    if (srv->fetcher.joinable()) srv->fetcher.join();
    if (srv->fetcher2.joinable()) srv->fetcher2.join();
    for (auto &kv : srv->reqs) {
        pgs_result_free(&kv.second->res);
        delete kv.second->pr;
        delete kv.second;
    }
    for (auto e : srv->lane_done)
        if (e) cudaEventDestroy(e);
    if (srv->fetch_stream) cudaStreamDestroy(srv->fetch_stream);
    if (srv->fetch_stream2) cudaStreamDestroy(srv->fetch_stream2);
    if (srv->up_stream) cudaStreamDestroy(srv->up_stream);
    if (srv->staged_ready) cudaEventDestroy(srv->staged_ready);
    for (auto &kv : srv->kcache) kentry_free(kv.second);
    for (auto &ws : srv->wins) {
        ws.r2.release();
        ws.full.release();
        if (ws.ready) cudaEventDestroy(ws.ready);
    }
    delete srv;
    return PGS_OK;
}

}  // extern "C"

namespace pgh {

void batch_state_destroy(pgs_ctx *ctx) {
    for (Lane *l : ctx->lanes) {
        cudaStreamSynchronize(l->stream);
        delete l;
    }
    ctx->lanes.clear();
    delete ctx->table;
    ctx->table = nullptr;
}

}  // namespace pgh
