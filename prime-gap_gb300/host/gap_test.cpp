// gap_test -- drop-in for the reference's probable-prime gap testers
// (gap_test_simple.cpp, gap_test_gpu.cu) on one GB300 through libpgsieve.
//
// Same flags and output as gap_test_simple: the unknowns file named by -u (or
// by -p/-d/--mstart/--minc/--sieve-length/--max-prime) is parsed on the device
// (pgs_parse_unknowns), every m's previous and next probable primes are found
// on the device (pgs_prp_gaps: each side's unknowns nearest first, then past
// the sieve length), and the gaps above --min-merit and the periodic stats
// lines are printed as gap_test_simple.cpp:107-199 and
// StatsCounters::process_results / possible_print_stats
// (gap_test_common.cpp:29-124) print them.  --one-side-skip applies
// gap_test_gpu's rule (gap_test_gpu.cu:570-596): the next side of an m is not
// searched when its previous gap's merit is below min_merit/2 - 2.
// The probable-prime test is gap_test_gpu's (base 2); gap_test_simple uses
// GMP's mpz_probab_prime_p, which differs only on base-2 strong pseudoprimes.
// Not printed: the GMP version line and prob_prime_and_stats' block of the
// reference's default verbosity (2); with -q the output matches line by line.
#include <cassert>
#include <chrono>
#include <clocale>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "cli_common.h"
#include "pgsieve.h"

namespace {

using namespace pgcli;

void show_usage(const char *name) {
    printf("Usage: %s\n", name);
    printf("[REQUIRED]\n  -p <p>\n  -d <p>\n  --mstart <start>\n  --minc   <int>\nOR\n");
    printf("  -u, --unknown-filename <filename>\n");
    printf("    parse p, d, mstart, minc, sieve-length, max-prime from filename\n\n");
    printf("[OPTIONALLY]\n  --min-merit <min_merit>\n    only display prime gaps with merit >= min_merit\n");
    printf("  --mskip <start at this m>\n  --one-side-skip\n");
    printf("    skip the next side when the previous gap's merit is below min_merit/2 - 2\n\n");
    printf("[OPTIONAL]\n  -q, --quiet\n  -h, --help\n\n");
    printf("tests the unknowns of (mstart + mi) * p#/d, mi <= minc for prime gaps\n");
}

// Args::guess_compression (gap_common.cpp:752-800) on the file's bytes.
int guess_compression(const Config &c, const std::string &text) {
    long long mtest = -1;
    sscanf(text.c_str(), "%lld", &mtest);
    assert(mtest >= 0);
    long long m = (long long)c.mstart;
    for (; gcd_u64(m, c.d) > 1; m++) {
    }
    if (m != mtest) {
        printf("\nfile format has changed,\n");
        printf("lines should start with <mstart + mi> not <mi>\n");
        printf("\texpected: %lld found: %lld\n", m, mtest);
        printf("you can add <mstart> to each line, recreate, or git checkout 74241f7c\n");
        printf("Sorry\n");
        exit(1);
    }
    const std::string t = text.substr(0, 99);
    for (size_t i = 0; i + 1 < t.size(); i++)
        if (t[i] == '|') {
            assert(i + 1 < t.size());
            if (t[i + 1] == '|') return 2;
            break;
        }
    bool has_space = false, has_high_range = false;
    for (size_t i = 50; i + 1 < t.size(); i++) {
        has_space |= t[i] == ' ' && t[i + 1] != '|' && t[i - 1] != '|';
        has_high_range |= t[i] > '9';
    }
    assert(has_space ^ has_high_range);
    return has_high_range ? 1 : 0;
}

// StatsCounters (gap_test_common.h:30-80, gap_test_common.cpp:29-124)
struct Stats {
    std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
    uint32_t s_tests = 0;
    size_t s_total_unknown = 0, s_t_unk_prev = 0, s_t_unk_next = 0, s_total_prp_tests = 0;
    size_t s_skips_after_one_side = 0, s_gap_out_of_sieve_prev = 0, s_gap_out_of_sieve_next = 0;
    float s_best_merit_interval = 0;
    size_t s_best_merit_interval_m = 0;
    float s_tests_per_second = 0;

    bool possible_print_stats(const Config &c, long m, bool is_last, size_t unknown_l, size_t unknown_u,
                              int prev_p, int next_p) {
        size_t print_interval = 1800 * s_tests_per_second;
        if (print_interval > 10000) print_interval -= (print_interval % 10000);
        bool is_power_print = (s_tests == 1);
        for (long p = 10; p <= s_tests; p *= 10)
            is_power_print |= (s_tests == p) || (s_tests == 3 * p) || (s_tests == 5 * p);
        if (!(is_last || is_power_print || (print_interval > 0 && s_tests % print_interval == 0))) return false;
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        s_tests_per_second = s_tests / secs;
        if ((c.verbose + is_last) >= 1) {
            printf("\tm=%ld %4ld <- unknowns -> %-4ld\t%4d <- gap -> %-4d\n", m, (long)unknown_l, (long)unknown_u,
                   prev_p, next_p);
            if (s_tests > secs)
                printf("\t    tests     %-10d (%.2f/sec)  %.0f seconds elapsed\n", s_tests, s_tests / secs, secs);
            else
                printf("\t    tests     %-10d (%.2f secs/test)  %.0f seconds elapsed\n", s_tests, secs / s_tests,
                       secs);
            printf("\t    unknowns  %-10ld (avg: %.2f), %.2f%% composite  %.2f%% <- %% -> %.2f%%\n",
                   (long)s_total_unknown, s_total_unknown / ((double)s_tests),
                   100.0 * (1 - s_total_unknown / ((2.0 * c.sieve_length + 1) * s_tests)),
                   100.0 * s_t_unk_prev / s_total_unknown, 100.0 * s_t_unk_next / s_total_unknown);
            printf("\t    prp tests %-10ld (avg: %.2f) (%.1f tests/sec)\n", (long)s_total_prp_tests,
                   s_total_prp_tests / (float)s_tests, s_total_prp_tests / secs);
            if (c.verbose >= 2) {
                if (s_skips_after_one_side)
                    printf("\t    only prev_prime %ld (%.2f%%)\n", (long)s_skips_after_one_side,
                           100.0 * s_skips_after_one_side / s_tests);
                if (s_gap_out_of_sieve_prev + s_gap_out_of_sieve_next > 0)
                    printf("\t    fallback prev_gap %ld (%.2f%%), next_gap %ld (%.2f%%)\n",
                           (long)s_gap_out_of_sieve_prev, 100.0 * s_gap_out_of_sieve_prev / s_tests,
                           (long)s_gap_out_of_sieve_next, 100.0 * s_gap_out_of_sieve_next / s_tests);
                printf("\t    best merit this interval: %.3f (at m=%ld)\n", s_best_merit_interval,
                       (long)s_best_merit_interval_m);
            }
        }
        return true;
    }

    void process_results(const Config &c, long m, bool is_last, size_t unknown_l, size_t unknown_u, int prev_p,
                         int next_p, int p_tests, int n_tests, float merit) {
        s_tests += 1;
        s_total_unknown += unknown_l + unknown_u;
        s_t_unk_prev += unknown_l;
        s_t_unk_next += unknown_u;
        s_total_prp_tests += p_tests + n_tests;
        if (merit > s_best_merit_interval) {
            s_best_merit_interval = merit;
            s_best_merit_interval_m = m;
        }
        if (possible_print_stats(c, m, is_last, unknown_l, unknown_u, prev_p, next_p)) {
            s_best_merit_interval = 0;
            s_best_merit_interval_m = 0;
        }
    }
};

}  // namespace

int main(int argc, char **argv) {
    bool one_side_skip = false;
    std::vector<char *> args;
    for (int i = 0; i < argc; i++) {
        if (i > 0 && strcmp(argv[i], "--one-side-skip") == 0) one_side_skip = true;
        else args.push_back(argv[i]);
    }
    Config c = argparse((int)args.size(), args.data(), show_usage);
    if (c.valid == 0) {
        show_usage(argv[0]);
        return 1;
    }
    if (c.sieve_length == 0) {
        printf("Must set sieve-length for %s\n", argv[0]);
        show_usage(argv[0]);
        return 1;
    }
    setlocale(LC_NUMERIC, "");
    if (c.verbose >= 0) {
        printf("\n");
        printf("Testing m * %d#/%d, m = %ld + [0, %'ld)\n", c.p, c.d, (long)c.mstart, (long)c.minc);
    }
    if (c.mskip > 0) {
        printf("\tskipping m < %'ld\n", (long)c.mskip);
        assert(c.mskip >= c.mstart);
        assert(c.mskip < (c.mstart + c.minc));
    }
    setlocale(LC_NUMERIC, "C");

    const std::string fn = gen_unknown_fn(c);
    if (c.verbose >= 1) printf("\nReading unknowns from '%s'\n", fn.c_str());
    std::string text;
    {
        std::ifstream f(fn, std::ios::in | std::ios::binary);
        assert(f.is_open());  // Can't open save_unknowns file
        assert(f.good());
        text.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    c.compression = guess_compression(c, text);

    // prime_gap_test (gap_test_simple.cpp:107-199)
    const double K_log = k_log(build_k(c.p, c.d));
    {
        const float m_log = log(c.mstart);
        if (c.verbose >= 1)
            printf("Min Gap ~= %d (for merit > %.1f)\n", (int)(c.min_merit * (K_log + m_log)), c.min_merit);
    }
    uint64_t valid_ms = 0;
    for (uint64_t mi = 0; mi < c.minc; mi++)
        if (gcd_u64(c.mstart + mi, c.d) == 1) valid_ms++;
    assert(valid_ms > 0);
    const uint64_t first_mi = 0;  // the reference's search loop for it never advances
    uint64_t last_mi = c.minc - 1;
    for (; last_mi > 0 && gcd_u64(c.mstart + last_mi, c.d) > 1; last_mi--) {
    }
    assert(last_mi > 0 && last_mi < c.minc);
    if (c.verbose >= 1)
        printf("\n%ld tests M_start(%ld) + mi(%ld to %ld)\n\n", (long)valid_ms, (long)c.mstart, (long)first_mi,
               (long)last_mi);

    pgs_ctx *ctx = nullptr;
    if (pgs_create(0, &ctx) != PGS_OK) {
        printf("no CUDA device available\n");
        return 1;
    }
    pgs_job job{c.p, c.d, c.mstart, c.minc, c.sieve_length, c.max_prime, c.compression, 0};
    pgs_unknowns u;
    if (pgs_parse_unknowns(ctx, &job, text.data(), text.size(), &u) != PGS_OK) {
        printf("can't parse '%s': %s\n", fn.c_str(), pgs_last_error(ctx));
        pgs_destroy(ctx);
        return 1;
    }
    // rows below --mskip are neither tested nor counted
    uint64_t first = 0;
    while (first < u.rows && u.m[first] < c.mskip) first++;
    pgs_unknowns view = u;
    view.rows = u.rows - first;
    view.m += first;
    view.start += first;
    view.n_prev += first;
    view.n_next += first;
    std::vector<pgs_gap_result> gaps(view.rows);
    pgs_gap_params gp{c.p, c.d, c.sieve_length, c.min_merit, one_side_skip ? 1 : 0};
    if (view.rows && pgs_prp_gaps(ctx, &gp, &view, gaps.data(), nullptr) != PGS_OK) {
        printf("gap search failed: %s\n", pgs_last_error(ctx));
        pgs_unknowns_free(&u);
        pgs_destroy(ctx);
        return 1;
    }
    Stats stats;  // rates and elapsed times count from here: the search is done
    for (uint64_t i = 0; i < view.rows; i++) {
        const long m = (long)view.m[i];
        const pgs_gap_result &g = gaps[i];
        const size_t unknown_l = view.n_prev[i], unknown_u = view.n_next[i];
        const bool is_last = (uint64_t)(m - (long)c.mstart) == last_mi;
        if (one_side_skip) {  // gap_test_gpu's counters
            stats.s_gap_out_of_sieve_prev += (g.flags & 1) ? 1 : 0;
            stats.s_gap_out_of_sieve_next += (g.flags & 2) ? 1 : 0;
        }
        if (g.flags & 4) {  // next side skipped: counted with the previous gap's merit
            stats.s_skips_after_one_side += 1;
            const float prev_merit = g.prev_p / (K_log + log(m));
            stats.process_results(c, m, is_last, unknown_l, unknown_u, g.prev_p, g.next_p, g.p_tests, g.n_tests,
                                  prev_merit);
            continue;
        }
        assert(g.prev_p > 0 && g.next_p > 0);
        const int gap = g.next_p + g.prev_p;
        const float merit = gap / (K_log + log(m));
        if (merit > c.min_merit)
            printf("%-5d %.4f  %ld * %ld#/%ld -%d to +%d\n", gap, merit, m, (long)c.p, (long)c.d, g.prev_p,
                   g.next_p);
        stats.process_results(c, m, is_last, unknown_l, unknown_u, g.prev_p, g.next_p, g.p_tests + g.n_tests, 0,
                              merit);
    }
    pgs_unknowns_free(&u);
    pgs_destroy(ctx);
    return 0;
}
