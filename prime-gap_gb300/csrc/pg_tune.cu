// Tuning: per job class, the launch knobs of the sieve kernels, chosen by
// timing candidates on the live device and cached per (device, class).
//
// The reference picks its phase thresholds per job with a hand cost model
// (calculate_thresholds_method2, gap_common.cpp:345-375); the output never
// depends on them.  Here the thresholds that decide which kernel walks a
// large prime (direct_steps, heavy_steps), the walk item size, the rows per
// CTA of the small-prime kernel, the chunks of the one-call text pipeline
// and the K mod p chain direction are the knobs, equally without effect on
// the output, and are measured instead of modelled.
#include <algorithm>
#include <cstring>

#include "pg_host.h"
#include "pg_tuning.h"

using namespace pgh;

namespace pgh {

pgs_tuning tuning_for(pgs_ctx *ctx, const pgs_job &job) {
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    auto it = ctx->tuning.find(pgt::tuning_class(job));
    return it == ctx->tuning.end() ? pgt::tuning_default() : it->second.t;
}

}  // namespace pgh

namespace {

// Median device time of `reps` runs of the prepared job (context locked);
// with pipeline, pgs_method2's rows/text/copy path (text freed).
int time_runs(pgs_ctx *ctx, pgs_prepared *pr, int reps, bool pipeline, double *ms) {
    cudaEvent_t a = nullptr, b = nullptr;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    std::vector<double> t;
    int rc = PGS_OK;
    for (int r = 0; r < reps && rc == PGS_OK; r++) {
        cudaError_t e = cudaEventRecord(a, ctx->stream);
        if (e) {
            rc = fail(ctx, e, "tune event");
            break;
        }
        HostText ht;
        rc = run_prepared(ctx, pr, 0, pipeline ? &ht : nullptr);
        if (rc) break;
        if ((e = cudaEventRecord(b, ctx->stream)) || (e = cudaEventSynchronize(b))) {
            rc = fail(ctx, e, "tune event");
            break;
        }
        float f = 0;
        cudaEventElapsedTime(&f, a, b);
        t.push_back(f);
        if (pipeline && ht.text) pinned_pool().put(ht.text, ht.cap);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return PGS_OK;
}

}  // namespace

extern "C" {

void pgs_tuning_default(pgs_tuning *out) {
    if (out) *out = pgt::tuning_default();
}

int pgs_tuning_class(const pgs_job *job, char *buf, size_t cap) {
    if (!job || !buf) return PGS_EINVAL;
    const std::string c = pgt::tuning_class(*job);
    if (c.size() + 1 > cap) return PGS_EINVAL;
    memcpy(buf, c.c_str(), c.size() + 1);
    return (int)c.size();
}

int pgs_tuning_set(pgs_ctx *ctx, const pgs_job *job, const pgs_tuning *t) {
    if (!ctx || !job || !t || !pgt::tuning_valid(*t)) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    pgt::Entry &e = ctx->tuning[pgt::tuning_class(*job)];
    e.t = *t;
    return PGS_OK;
}

int pgs_tuning_get(pgs_ctx *ctx, const pgs_job *job, pgs_tuning *out) {
    if (!ctx || !job || !out) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    auto it = ctx->tuning.find(pgt::tuning_class(*job));
    *out = it == ctx->tuning.end() ? pgt::tuning_default() : it->second.t;
    return it != ctx->tuning.end();
}

int pgs_tuning_load(pgs_ctx *ctx, const char *path) {
    if (!ctx || !path) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    const int n = pgt::load(path, ctx->device_name, ctx->tuning);
    if (n < 0) {
        ctx->err = std::string("cannot read tuning file ") + path;
        return PGS_EINVAL;
    }
    return n;
}

int pgs_tuning_save(pgs_ctx *ctx, const char *path) {
    if (!ctx || !path) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    const int n = pgt::save(path, ctx->device_name, ctx->tuning);
    if (n < 0) {
        ctx->err = std::string("cannot write tuning file ") + path;
        return PGS_EINVAL;
    }
    return n;
}

int pgs_tune(pgs_ctx *ctx, const pgs_job *job, int reps, pgs_tuning *out, double *ms_default, double *ms_tuned) {
    if (!ctx || !job || reps < 1) return PGS_EINVAL;
    pgs_prepared *pr = nullptr;
    int rc = pgs_prepare(ctx, job, &pr);
    if (rc) return rc;
    std::lock_guard<std::mutex> g(ctx->mu);
    pgs_tuning best = pgt::tuning_default();
    double t_def = 0, t_best = 0, t_pipe = 0;
    auto measure = [&](const pgs_tuning &t, bool pipeline, double *ms) {
        pr->tune = t;
        return time_runs(ctx, pr, reps, pipeline, ms);
    };
    rc = measure(best, false, &t_def);
    // warm-up effects land on the first candidate: measure the default twice
    if (!rc) rc = measure(best, false, &t_def);
    t_best = t_def;
    struct Knob {
        uint32_t pgs_tuning::*field;
        std::vector<uint32_t> values;
    };
    const std::vector<Knob> knobs = {
        {&pgs_tuning::large_form, {0, 1, 2, 3, 4, 5, 6, 7}},
        {&pgs_tuning::heavy_steps, {1024, 2048, 4096, 8192, 16384}},
        {&pgs_tuning::item_steps, {32, 64, 128}},
        {&pgs_tuning::direct_steps, {8, 16, 24, 32, 48}},
        {&pgs_tuning::rows_per_cta, {4, 8, 12, 16, 24, 32}},
        {&pgs_tuning::kmod_lsb_limbs, {8, 16, 24, 32, 48, 64, 1u << 20}},
    };
    for (const Knob &k : knobs) {
        if (rc) break;
        for (uint32_t v : k.values) {
            pgs_tuning c = best;
            c.*(k.field) = v;
            if (v == best.*(k.field) || !pgt::tuning_valid(c)) continue;
            double ms = 0;
            if ((rc = measure(c, false, &ms))) break;
            if (ms < t_best * 0.98) best = c, t_best = ms;
        }
    }
    // the one-call pipeline's chunks, timed through that pipeline
    if (!rc) rc = measure(best, true, &t_pipe);
    for (uint32_t v = 1; v <= 4 && !rc; v++) {
        if (v == best.text_chunks) continue;
        pgs_tuning c = best;
        c.text_chunks = v;
        double ms = 0;
        if ((rc = measure(c, true, &ms))) break;
        if (ms < t_pipe * 0.98) best = c, t_pipe = ms;
    }
    // confirm against the defaults, measured alternately: a pick that only
    // won on noise falls back to the defaults
    if (!rc) {
        std::vector<double> d, b;
        for (int r = 0; r < 3 && !rc; r++) {
            double x = 0, y = 0;
            if (!(rc = measure(pgt::tuning_default(), false, &x)) && !(rc = measure(best, false, &y)))
                d.push_back(x), b.push_back(y);
        }
        if (!rc) {
            std::sort(d.begin(), d.end());
            std::sort(b.begin(), b.end());
            t_def = d[1];
            t_best = b[1];
            if (t_best > t_def * 0.99) {
                const uint32_t chunks = best.text_chunks;
                best = pgt::tuning_default();
                best.text_chunks = chunks;  // measured on its own pipeline
                t_best = t_def;
            }
        }
    }
    if (!rc) {
        std::lock_guard<std::mutex> tg(ctx->tune_mu);
        pgt::Entry &e = ctx->tuning[pgt::tuning_class(*job)];
        e.t = best;
        e.ms_default = t_def;
        e.ms_tuned = t_best;
    }
    pgs_prepared_free(pr);
    if (rc) return rc;
    if (out) *out = best;
    if (ms_default) *ms_default = t_def;
    if (ms_tuned) *ms_tuned = t_best;
    return PGS_OK;
}

}  // extern "C"
