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
    CK(l->ctr.ensure(2 * sizeof(unsigned long long)));
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
        CK(pg::rows_extract(rd, rows_per_block(h.nb, h.job.compression), s));
        CK(pg::scan_u64(pr->row_bytes.as<uint64_t>(), pr->offsets.as<uint64_t>(), pr->misc.as<uint64_t>(),
                        rows, pr->scan_tmp.as<uint64_t>(), s));
        CK(pg::format_rows(rd, pr->offsets.as<uint64_t>(), pr->text.as<char>(), s));
        pr->launches += 5;
        pr->ran = true;
    }
    return PGS_OK;
}

int run_table_job(pgs_ctx *ctx, pgs_prepared *pr, Lane *lane) {
    return run_group(ctx, std::vector<pgs_prepared *>{pr}, lane, nullptr);
}

uint64_t job_cost(const HostJob &h) {
    const double lim = (double)h.prime_limit;
    const double primes = lim / std::log(std::max(lim, 3.0));
    return (uint64_t)(primes * ((double)h.klimbs.size() + 150.0) +
                      (double)h.valid_mi.size() * h.H * 2.0);
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

// Jobs with the same P form a group sharing K' = P#/L (L = lcm of their d)
// when every L/d fits 32 bits; otherwise jobs group by their exact K.
// Groups go longest first onto the least-loaded lane; the result is in that
// (launch) order.
std::vector<GroupPlan> plan_groups(const std::vector<const HostJob *> &hj, int lanes) {
    std::map<uint32_t, std::vector<int>> by_p;
    for (int i = 0; i < (int)hj.size(); i++) by_p[hj[i]->job.p].push_back(i);
    std::vector<GroupPlan> out;
    for (auto &kv : by_p) {
        uint64_t L = 1;
        bool ok = kv.second.size() > 1;
        for (int i : kv.second) {
            const uint64_t d = hj[i]->job.d;
            const uint64_t g = gcd64(L, d);
            if (L / g > (~0ull >> 1) / d) {
                ok = false;
                break;
            }
            L = L / g * d;
        }
        for (int i : kv.second) ok = ok && L / hj[i]->job.d <= 0xFFFFFFFFull;
        if (ok) {
            GroupPlan gp;
            gp.jobs = kv.second;
            gp.klimbs = primorial_quotient(kv.first, L);
            for (int i : kv.second) gp.kmul.push_back((uint32_t)(L / hj[i]->job.d));
            out.push_back(std::move(gp));
            continue;
        }
        std::map<uint32_t, GroupPlan> by_d;  // same K
        for (int i : kv.second) {
            GroupPlan &gp = by_d[hj[i]->job.d];
            gp.jobs.push_back(i);
            gp.kmul.push_back(1);
            gp.klimbs = hj[i]->klimbs;
        }
        for (auto &dg : by_d) out.push_back(std::move(dg.second));
    }
    for (GroupPlan &gp : out)
        for (int i : gp.jobs) gp.cost += job_cost(*hj[i]);
    std::sort(out.begin(), out.end(), [](const GroupPlan &a, const GroupPlan &b) { return a.cost > b.cost; });
    std::vector<uint64_t> load(lanes, 0);
    for (GroupPlan &gp : out) {
        gp.lane = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[gp.lane] += gp.cost;
    }
    return out;
}

// Device copies of the groups' K' limbs, packed; offsets per group.
cudaError_t upload_group_limbs(const std::vector<GroupPlan> &groups, DevBuf &buf,
                               std::vector<size_t> &offset, cudaStream_t s) {
    std::vector<uint32_t> all;
    offset.clear();
    for (const GroupPlan &gp : groups) {
        offset.push_back(all.size());
        all.insert(all.end(), gp.klimbs.begin(), gp.klimbs.end());
    }
    return upload(buf, all, s);
}

}  // namespace

struct pgs_batch {
    pgs_ctx *ctx = nullptr;
    std::vector<pgs_prepared *> jobs;
    std::vector<int> lane_of;
    std::vector<GroupPlan> groups;         // in launch order
    std::vector<size_t> group_urange;      // offset (words) of each group's hull ranges
    std::vector<size_t> group_limbs;       // offset of each group's K' limbs
    DevBuf urange, glimbs;
    int nlanes = 1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> joins;
};

namespace {

int launch_batch(pgs_ctx *ctx, pgs_batch *b) {
    Lane *l0 = ctx->lanes[0];
    CK(cudaEventRecord(b->fork, l0->stream));
    for (int l = 1; l < b->nlanes; l++) CK(cudaStreamWaitEvent(ctx->lanes[l]->stream, b->fork, 0));
    for (size_t g = 0; g < b->groups.size(); g++) {
        const GroupPlan &gp = b->groups[g];
        std::vector<pgs_prepared *> jobs;
        for (int j : gp.jobs) jobs.push_back(b->jobs[j]);
        int rc = run_group(ctx, jobs, ctx->lanes[gp.lane], b->urange.as<unsigned long long>() + b->group_urange[g],
                           b->glimbs.as<uint32_t>() + b->group_limbs[g], (int)gp.klimbs.size(), gp.kmul);
        if (rc) return rc;
    }
    for (int l = 1; l < b->nlanes; l++) {
        CK(cudaEventRecord(b->joins[l], ctx->lanes[l]->stream));
        CK(cudaStreamWaitEvent(l0->stream, b->joins[l], 0));
    }
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
    *out = nullptr;
    std::vector<HostJob> hj;
    int rc = derive_all(jobs, n, hj, true, ctx->err);
    if (rc) return rc;
    // cover every job: large primes up to the largest limit, small up to the largest S1
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
    std::vector<const HostJob *> hp;
    for (const HostJob &h : hj) hp.push_back(&h);
    b->groups = plan_groups(hp, L);
    const int G = (int)b->groups.size();
    b->lane_of.assign(n, 0);
    for (int g = 0; g < G; g++)
        for (int j : b->groups[g].jobs) b->lane_of[j] = b->groups[g].lane;
    b->glimbs.pool = &ctx->dpool;
    cudaError_t le = upload_group_limbs(b->groups, b->glimbs, b->group_limbs, ctx->stream);
    if (le != cudaSuccess) {
        pgs_batch_free(b);
        return fail(ctx, le, "batch group limbs");
    }
    for (int i = 0; i < n; i++) {
        pgs_prepared *pr = nullptr;
        rc = prepare_table_job(ctx, jobs[i], ctx->stream, &pr, &hj[i]);
        if (rc) {
            pgs_batch_free(b);
            return rc;
        }
        b->jobs.push_back(pr);
    }
    size_t words = 0;
    for (int g = 0; g < G; g++) {
        b->group_urange.push_back(words);
        words += 2 * ctx->table->windows.size();
    }
    b->urange.pool = &ctx->dpool;
    cudaError_t ue = b->urange.ensure(std::max<size_t>(words, 2) * 8);
    if (ue != cudaSuccess) {
        pgs_batch_free(b);
        return fail(ctx, ue, "batch ranges");
    }
    CK(cudaEventCreate(&b->t0));
    CK(cudaEventCreate(&b->t1));
    CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->joins.assign(L, nullptr);
    for (int l = 1; l < L; l++) CK(cudaEventCreateWithFlags(&b->joins[l], cudaEventDisableTiming));
    CK(cudaStreamSynchronize(ctx->stream));
    *out = b;
    return PGS_OK;
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
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->fork) cudaEventDestroy(b->fork);
    for (auto e : b->joins)
        if (e) cudaEventDestroy(e);
    for (auto *pr : b->jobs) delete pr;
    b->urange.release();
    b->glimbs.release();
    delete b;
}

// One pass, pipelined: host work (job tables) is done up front on several
// threads, each group's uploads go on the context stream and its kernels on
// its lane as soon as they are enqueued, and results are copied back group by
// group as each finishes, while the other lanes still compute.
int pgs_method2_batch(pgs_ctx *ctx, const pgs_job *jobs, int n, pgs_result *outs) {
    if (!ctx || !jobs || n <= 0 || !outs) return PGS_EINVAL;
    for (int i = 0; i < n; i++) memset(&outs[i], 0, sizeof(pgs_result));
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
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
    const int L = std::max(1, std::min(8, n));
    rc = ensure_lanes(ctx, L);
    if (rc) return rc;
    std::vector<const HostJob *> hp;
    for (const HostJob &h : hj) hp.push_back(&h);
    const std::vector<GroupPlan> groups = plan_groups(hp, L);
    const int G = (int)groups.size();
    const size_t nwin = ctx->table->windows.size();
    DevBuf urange, glimbs;
    urange.pool = glimbs.pool = &ctx->dpool;
    std::vector<size_t> limb_off;
    std::vector<pgs_prepared *> prs(n, nullptr);
    std::vector<cudaEvent_t> up_done(G, nullptr), done(G, nullptr);
    cudaStream_t up = ctx->stream;
    auto cleanup = [&] {
        for (Lane *l : ctx->lanes) cudaStreamSynchronize(l->stream);
        cudaStreamSynchronize(up);
        for (auto *pr : prs) delete pr;
        for (auto e : up_done)
            if (e) cudaEventDestroy(e);
        for (auto e : done)
            if (e) cudaEventDestroy(e);
        urange.release();
        glimbs.release();
    };
    cudaError_t e = urange.ensure(std::max<size_t>(2 * nwin * G, 2) * 8);
    if (e == cudaSuccess) e = upload_group_limbs(groups, glimbs, limb_off, up);
    for (int k = 0; k < G && e == cudaSuccess; k++) {
        e = cudaEventCreateWithFlags(&up_done[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        cleanup();
        return fail(ctx, e, "batch setup");
    }
    for (int grp = 0; grp < G && rc == PGS_OK; grp++) {
        const GroupPlan &gp = groups[grp];
        Lane *lane = ctx->lanes[gp.lane];
        std::vector<pgs_prepared *> members;
        for (int j : gp.jobs) {
            rc = prepare_table_job(ctx, jobs[j], up, &prs[j], &hj[j]);
            if (rc) break;
            members.push_back(prs[j]);
        }
        if (rc) break;
        if ((e = cudaEventRecord(up_done[grp], up)) || (e = cudaStreamWaitEvent(lane->stream, up_done[grp], 0))) {
            rc = fail(ctx, e, "batch upload order");
            break;
        }
        rc = run_group(ctx, members, lane, urange.as<unsigned long long>() + 2 * nwin * grp,
                       glimbs.as<uint32_t>() + limb_off[grp], (int)gp.klimbs.size(), gp.kmul);
        if (rc == PGS_OK && (e = cudaEventRecord(done[grp], lane->stream))) rc = fail(ctx, e, "batch event");
    }
    // results, group by group in launch order, on the upload stream
    for (int grp = 0; grp < G && rc == PGS_OK; grp++) {
        if ((e = cudaStreamWaitEvent(up, done[grp], 0))) {
            rc = fail(ctx, e, "batch fetch order");
            break;
        }
        for (int j : groups[grp].jobs) {
            rc = fetch_job(ctx, prs[j], up, &outs[j]);
            if (rc) break;
        }
    }
    if (rc != PGS_OK)
        for (int i = 0; i < n; i++) pgs_result_free(&outs[i]);
    cleanup();
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
