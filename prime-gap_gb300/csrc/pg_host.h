// Host-side internals of libpgsieve shared by the plain path (pg_api.cu) and
// the batched / served paths (pg_batch.cu): derived job tables, device and
// pinned buffer pools, the context and the prepared-job objects.
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "pg_internal.h"
#include "pg_tuning.h"
#include "pgsieve.h"

namespace pgh {

constexpr uint64_t kWindowSpan = 1ull << 30;

bool is_prime_u64(uint64_t n);
uint64_t next_prime_above(uint64_t n);
std::vector<uint32_t> primes_upto(uint32_t n);
uint32_t ndigits(uint64_t v);

struct HostJob {
    pgs_job job{};
    std::vector<uint32_t> klimbs;
    uint32_t kbits = 0;
    std::vector<uint32_t> valid_mi;
    std::vector<uint32_t> dist;
    // the live offsets over the row bitmap's index (x - x_par) / 2, nb bits
    std::vector<uint32_t> live;
    std::vector<uint32_t> dq;  // odd primes dividing d
    // valid-m bitmask over walk indices j and live-offset bitmask over walk
    // residues y (pg_host.cu), as {bits, set bits before the word} pairs
    std::vector<uint32_t> mmask, ymask;
    uint32_t x_par = 0, nb = 0, H = 0, Hp = 0, pitch = 0;
    uint32_t y_lo = 0;  // walk residues y >= y_lo are offsets below SL
    uint64_t coprime_x = 0;
    uint64_t small_threshold = 0, medium_threshold = 0, prime_limit = 0;
    uint64_t s1 = 0;
    uint64_t primes_to_P = 0;  // primes <= min(P, prime_limit), 2 included
    pg::WalkParams walk{};
    std::string filename;
};

// Validate a job (the reference's argparse/main rules) and derive its tables;
// tables=false stops after the scalar parameters.
int derive(const pgs_job &j, HostJob &h, std::string &err, bool tables);

// Device allocations recycled across jobs on one context: a job's buffers
// (several GB for the larger configs) are returned here instead of freed, so
// repeated jobs pay no cudaMalloc/cudaFree.
// Allocation size classes: n rounded up to one of 8 steps per power of two
// (at most 12.5 % over), so buffers freed by one job fit the next job's
// slightly different sizes and pools stop growing after a few jobs.
inline size_t size_class(size_t n) {
    if (n <= 4096) return 4096;
    const int b = 63 - __builtin_clzll((unsigned long long)(n - 1));  // n - 1 < 2^(b+1)
    const size_t step = (size_t)1 << (b - 2 > 12 ? b - 2 : 12);
    return (n + step - 1) / step * step;
}

struct DevicePool {
    std::mutex mu;
    std::vector<std::pair<void *, size_t>> free_list;
    double alloc_s = 0;  // time spent in cudaMalloc
    uint64_t allocs = 0;
    cudaError_t get(size_t n, void **p, size_t *cap) {
        n = size_class(n);
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
        const auto t0 = std::chrono::steady_clock::now();
        cudaError_t e = cudaMalloc(p, n);
        if (e == cudaErrorMemoryAllocation) {
            trim();  // give cached blocks back and retry once
            e = cudaMalloc(p, n);
        }
        if (e == cudaSuccess) {
            *cap = n;
            std::lock_guard<std::mutex> g(mu);
            alloc_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            allocs++;
        }
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
    double alloc_s = 0;  // time spent in cudaMallocHost
    uint64_t allocs = 0;
    char *get(size_t n, size_t *cap) {
        {
            std::lock_guard<std::mutex> g(mu);
            size_t best = (size_t)-1;
            for (size_t i = 0; i < free_list.size(); i++)
                if (free_list[i].second >= n &&
                    (best == (size_t)-1 || free_list[i].second < free_list[best].second))
                    best = i;
            if (best != (size_t)-1) {
                auto e = free_list[best];
                free_list.erase(free_list.begin() + best);
                *cap = e.second;
                return e.first;
            }
        }
        char *p = nullptr;
        const size_t want = size_class(n);
        const auto t0 = std::chrono::steady_clock::now();
        if (cudaMallocHost(&p, want) != cudaSuccess) return nullptr;
        std::lock_guard<std::mutex> g(mu);
        alloc_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        allocs++;
        *cap = want;
        return p;
    }
    void put(char *p, size_t cap) {
        std::lock_guard<std::mutex> g(mu);
        free_list.push_back({p, cap});
    }
};

PinnedPool &pinned_pool();

struct PinnedOwner {
    size_t cap;
};

struct Window {
    uint64_t lo, hi, bound;
    bool wide;
};

}  // namespace pgh

struct PrimeTable;
struct Lane;

// Chunks of rows whose text is copied to the host while later chunks run.
constexpr int kTextChunks = 4;

struct pgs_ctx {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t copy = nullptr;  // text copies to the host beside the job's kernels
    // one stream per chunk of rows, earlier chunks at higher priority
    cudaStream_t chunk[kTextChunks] = {};
    std::mutex mu;
    std::string err;
    pg::BasePrimes base;
    pgh::DevBuf win_off, win_r, win_t0, large_ctr, heavy, walks;
    // the next window's primes and K mod p, made on `aux` while the large
    // primes of the current window run on the job's stream
    pgh::DevBuf win_off2, win_r2, win_t02;
    cudaStream_t aux = nullptr;
    pgh::DevicePool dpool;
    // batched / served paths (pg_batch.cu)
    PrimeTable *table = nullptr;
    std::vector<Lane *> lanes;
    // tuning by class (pg_tune.cu); device name for the cache file
    std::mutex tune_mu;
    std::map<std::string, pgt::Entry> tuning;
    std::string device_name;
};

struct pgs_prepared {
    pgs_ctx *ctx = nullptr;
    pgh::HostJob hj;
    pgs_tuning tune{24, 64, 4096, 16, 4, 32, 0};  // the job's class tuning (defaults)
    std::vector<pgh::Window> windows;
    uint64_t sp_lo = 0, sp_hi = 0, sp_bound = 0;
    uint64_t text_cap = 0;
    // resident-table jobs (pg_batch.cu): small primes are table entries
    // [tbl_a, tbl_b), large primes come from the table windows listed
    bool table_mode = false;
    uint64_t tbl_a = 0, tbl_b = 0;
    std::vector<int> tbl_windows;
    // primes above the small phase that the job sieves, when the host knows
    // them (the batch finds every range at prepare time); ~0 when they are
    // read from the job's range words on the device
    uint64_t large_primes = ~0ull;
    size_t footprint = 0;  // device bytes held by this job
    uint64_t win_bound = 0;
    pgh::DevBuf klimbs, valid_mi, dist, live, dq, dr, comp, sp, sr, sp_t0, mmask, ymask;
    pgh::DevBuf lists, counts, row_bytes, offsets, scan_tmp, misc, text;
    pgh::DevBuf row_count, row_off, bucket;  // the per-m path (method1)
    std::vector<cudaEvent_t> events;
    std::vector<std::pair<int, std::pair<int, int>>> spans;  // stage, (ev a, ev b)
    double ms_setup = 0;
    uint64_t launches = 0;
    bool ran = false;
    std::vector<pgh::DevBuf *> all() {
        return {&klimbs, &valid_mi, &dist,  &live,     &dq,        &dr,       &comp,
                &sp,     &sr,       &sp_t0, &lists,    &counts,    &row_bytes, &offsets,
                &scan_tmp, &misc,   &text,  &mmask,    &ymask,     &row_count, &row_off,
                &bucket};
    }
    char *stage = nullptr;  // pinned staging block of the table uploads
    size_t stage_cap = 0;
    ~pgs_prepared() {
        for (auto e : events) cudaEventDestroy(e);
        for (pgh::DevBuf *b : all()) b->release();
        if (stage) pgh::pinned_pool().put(stage, stage_cap);
    }
};

namespace pgh {

int fail(pgs_ctx *ctx, cudaError_t e, const char *what);

// A job's unknown lists as one packed device block: m (u64), start (u64),
// n_prev, n_next (u32) per row, then the distances (u32), as pgs_unknowns.
struct PackedLists {
    DevBuf block;
    uint64_t rows = 0, total = 0;
    uint64_t *m = nullptr, *start = nullptr;
    uint32_t *n_prev = nullptr, *n_next = nullptr, *dist = nullptr;
};
// Carves pk.block (allocated for rows and max_total distances) into its pieces.
cudaError_t packed_alloc(PackedLists &pk, uint64_t rows, uint64_t max_total);
// A sieved job's lists on the device (pg_unknowns.cu); the caller releases
// pk.block after the stream is done with it.
int job_lists_device(pgs_ctx *ctx, pgs_prepared *pr, cudaStream_t s, PackedLists &pk);

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

pg::JobDev job_dev(pgs_prepared *pr);
// The tuning jobs of this class get on the context (defaults when untuned).
pgs_tuning tuning_for(pgs_ctx *ctx, const pgs_job &job);
pg::RowsDev rows_dev(pgs_prepared *pr);
uint32_t rows_per_block(uint32_t nb, int compression, uint32_t cap = 16);

// The job's host tables (K limbs, row/column maps, valid m, distances, primes
// of d, masks) to their device buffers, through one pinned staging block:
// a copy from pageable memory is staged by CUDA and waits for it.
cudaError_t upload_tables(pgs_prepared *pr, cudaStream_t s);

// Text already copied to pinned host memory (the pipelined one-call path).
struct HostText {
    char *text = nullptr;
    size_t cap = 0;       // pinned pool capacity
    uint64_t total = 0;   // bytes
    float ms_d2h = 0;
};
// A finished job's result: its text copied to pinned host memory, or the
// text given, and its counts and stage times (no context lock).
int fetch_job(pgs_ctx *ctx, pgs_prepared *pr, cudaStream_t s, pgs_result *out,
              const HostText *given = nullptr);
// One run of a prepared job with the context locked (the body of pgs_run;
// with `sink`, pgs_method2's pipelined rows, text and copy to the host).
int run_prepared(pgs_ctx *ctx, pgs_prepared *pr, int record_stages, HostText *sink);
// Number of {begin, end} prime ranges in a prepared job's misc buffer.
size_t job_ranges(const pgs_prepared *pr);
// Free the resident prime table and the lanes (pg_batch.cu).
void batch_state_destroy(pgs_ctx *ctx);

}  // namespace pgh
