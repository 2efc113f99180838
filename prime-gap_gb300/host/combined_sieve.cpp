// combined_sieve -- drop-in replacement for the reference's combined_sieve
// process (method2 path) running on one GB300 through libpgsieve.
//
// Same flags and unknowns-file name as the reference: Args::argparse
// (gap_common.cpp:805-1099), Args::gen_unknown_fn (gap_common.cpp:732-749) and
// main()'s validation (combined_sieve.cpp:74-157).  Writes the same bytes to
// unknowns/<P>_<d>_<mstart>_<minc>_s<SL>_l<MP>M.txt and records the run in the
// search database's `range` table like insert_range_db
// (combined_sieve.cpp:347-380).  Exit codes: 0 ok, 1 invalid arguments or
// failed run (the reference's exit(1)).
//
// --method1 runs the per-m path (pgs_method1: each m's large-prime marks
// from its own bucket, as the reference's prime_gap_search takes them from
// its next-m queue) and writes the same bytes (the reference checks the two
// methods against each other, misc/tests.sh:62-67) under the .m1.txt name.
// set_defaults (combined_sieve.cpp:160-344) runs as in the reference: the d
// optimizer for d % 4 == 0 (count_K_d statistics, gap_common.cpp:455-571,
// then exit 0), the automatic sieve length and the automatic max_prime.
#include <dlfcn.h>
#include <getopt.h>
#include <libgen.h>

#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "cli_common.h"
#include "pgsieve.h"

namespace {

using namespace pgcli;

// prob_prime_coprime (gap_common.cpp:615-625)
double prob_prime_coprime(const Config &c) {
    const double N_log = k_log(build_k(c.p, c.d)) + std::log((double)c.mstart);
    double prob = 1 / N_log - 1 / (N_log * N_log);
    for (uint32_t q : primes_upto(c.p)) prob /= (1 - 1.0 / q);
    return prob;
}

// count_K_d (gap_common.cpp:455-571): average expected gap, coprime
// offsets per side and the chance a side has no prime within SL, over the
// first (up to 5000) valid m.
std::tuple<double, uint32_t, double, double> count_K_d(const Config &c) {
    const uint64_t d = c.d;
    const uint64_t K_mod_d = k_mod(build_k(c.p, c.d), c.d);
    const std::vector<uint32_t> P_primes = primes_upto(c.p);
    assert(P_primes.back() == c.p);
    const double prob_prime_adj = prob_prime_coprime(c);
    std::vector<uint32_t> D_primes;
    for (uint32_t q : P_primes)
        if (d % q == 0) D_primes.push_back(q);
    const size_t sl = c.sieve_length, length = 2 * sl + 1;
    std::vector<char> compositeK(length, 0), composite(length);
    for (uint32_t q : P_primes)
        if (d % q != 0)
            for (size_t x = sl % q; x < length; x += q) compositeK[x] = 1;
    double expected_length = 0, remaining_prob = 0;
    size_t expected_count = 0, m_count = 0;
    const uint64_t intervals = std::min<uint64_t>(d, 5000);
    for (uint64_t m = c.mstart; m_count < intervals; m++) {
        if (m >= c.mstart + c.minc) break;
        if (d > 1 && gcd_u64(m, d) > 1) continue;
        m_count++;
        composite = compositeK;
        for (uint32_t q : D_primes) {
            assert(K_mod_d % q != 0);
            const uint64_t first = (q - (((m % q) * (K_mod_d % q) + q - (sl % q)) % q)) % q;
            for (size_t x = first; x < length; x += q) composite[x] = 1;
        }
        for (int dir = -1; dir <= 1; dir += 2) {
            double expected = 0, prob = 1.0;
            for (int x = 0; (size_t)x <= sl; x++) {
                if (!composite[sl + dir * x]) {
                    expected += x * prob * prob_prime_adj;
                    prob *= 1 - prob_prime_adj;
                    expected_count += 1;
                }
            }
            expected += sl * prob;
            expected_length += expected;
            remaining_prob += prob;
        }
    }
    return {expected_length / m_count, (uint32_t)(expected_count / (m_count * 2)),
            remaining_prob / (m_count * 2), prob_prime_adj};
}

// The d optimizer (combined_sieve.cpp:166-209): for d = 4 * large_prime (or
// 4), statistics of d = lp * q# for lp in {1, large prime}; exits 0.
[[noreturn]] void d_optimizer(Config c) {
    c.sieve_length = c.p * c.min_merit;
    c.mstart = 1;
    c.d /= 4;
    const std::vector<uint32_t> P_primes = primes_upto(c.p);
    const uint32_t rand_prime = P_primes[P_primes.size() - 2 - (rand() % 10)];
    const uint32_t large_p = c.d > 1 ? c.d : rand_prime;
    assert(is_prime_brute(large_p));
    printf("d optimizer for P = %d# | large prime=%d | SL=%d (%.1f merit)\n", c.p, large_p, c.sieve_length,
           c.min_merit);
    const uint32_t primes[] = {1, 2, 3, 5, 7, 11, 13, 17, 19, 23};
    for (uint32_t lp : {1u, large_p}) {
        c.d = lp;
        for (uint32_t q : primes) {
            if (q != 1 && c.d % q == 0) continue;
            if (__builtin_umul_overflow(c.d, q, &c.d)) break;
            c.minc = std::min(c.d, 20000U);
            const auto expected = count_K_d(c);
            printf("Optimizing | d = %5d * %2d# | %d remaining, %5.0f avg gap | SL insufficient %.3f%% of time\n",
                   lp, q, std::get<1>(expected), std::get<0>(expected), 100 * std::get<2>(expected));
        }
    }
    exit(0);
}

// The automatic sieve length (combined_sieve.cpp:224-308): the smallest SL
// at which, for the worst (m*K) mod d of the range, the chance that no
// coprime offset in (0, SL] is prime falls to 0.8 %.
uint32_t auto_sieve_length(const Config &c) {
    const double prob_prime_coprime_P = prob_prime_coprime(c);
    std::vector<uint32_t> K_primes;
    for (uint32_t q : primes_upto(c.p))
        if (c.d % q != 0) K_primes.push_back(q);
    assert(c.p >= 503);
    assert(c.d <= 30030);
    const uint32_t base = k_mod(build_k(c.p, c.d), c.d);
    std::vector<uint32_t> count_by_mod_d(c.d, 0);
    for (uint64_t mi = 0; mi < c.minc; mi++) {
        const uint64_t m = c.mstart + mi;
        if (gcd_u64(m, c.d) == 1) {
            const uint32_t center = (uint32_t)(((unsigned __int128)m * base) % c.d);
            const uint32_t center_down = (c.d - center) % c.d;
            count_by_mod_d[center] += 1;
            count_by_mod_d[center_down] += 1;
        }
    }
    std::map<uint32_t, uint32_t> coprime_by_mod_d;
    for (size_t i = 0; i < c.d; i++)
        if (count_by_mod_d[i] > 0) coprime_by_mod_d[(uint32_t)i] = 0;
    for (size_t tSL = 1;; tSL += 1) {
        bool any_divisible = false;
        for (uint32_t q : K_primes)
            if (tSL % q == 0) {
                any_divisible = true;
                break;
            }
        if (any_divisible) continue;
        for (auto &cc : coprime_by_mod_d)
            if (gcd_u64(cc.first + tSL, c.d) == 1) cc.second += 1;
        uint32_t min_coprime = (uint32_t)tSL;
        for (auto &cc : coprime_by_mod_d) min_coprime = std::min(min_coprime, cc.second);
        const double prob_gap_shorter = std::pow(1 - prob_prime_coprime_P, min_coprime);
        if (prob_gap_shorter <= 0.008) {
            printf("AUTO SET: sieve length: %ld (coprime: %d, prob_gap longer %.2f%%)\n", (long)tSL, min_coprime,
                   100 * prob_gap_shorter);
            return (uint32_t)tSL;
        }
    }
}

void show_usage(const char *name) {
    printf("Usage: %s\n", name);
    printf("[REQUIRED]\n  -p <p>\n  -d <p>\n  --mstart <start>\n  --minc   <int>\nOR\n");
    printf("  -u, --unknown-filename <filename>\n");
    printf("    parse p, d, mstart, minc, sieve-length, max-prime from filename\n\n");
    printf("[OPTIONALLY]\n  -t, --threads N\n  --min-merit <min_merit>\n");
    printf("  --sieve-length\n    how large the positive/negative sieve arrays should be\n");
    printf("  --max-prime\n    use primes <= max-prime (in millions) for checking composite\n\n");
    printf("  --save-unknowns\n  --rle\n  --bitcompress\n  --maxmem <max memory in GB>\n\n");
    printf("[OPTIONAL]\n  --search-db\n  --prime-gaps-db\n\n  -q, --quiet\n  -h, --help\n\n");
    printf("calculates prime_gaps for (mstart + mi) * p#/d, mi <= minc \n");
}

// config hash used as the range id (gap_common.cpp:1112-1121)
uint64_t config_hash(const Config &c) {
    uint64_t hash = c.mstart;
    hash = hash * 31 + c.minc;
    hash = hash * 31 + c.p;
    hash = hash * 31 + c.d;
    hash = hash * 31 + c.sieve_length;
    hash = hash * 31 + c.max_prime;
    return hash;
}

// insert_range_db (combined_sieve.cpp:347-380) through the system sqlite3.
int insert_range_db(const Config &c, long num_rows, float time_sieve) {
    require_file(c.search_db.c_str());
    void *h = dlopen("libsqlite3.so.0", RTLD_NOW);
    if (!h) {
        printf("\nrange INSERT failed: libsqlite3.so.0 not available\n");
        return 1;
    }
    typedef int (*open_t)(const char *, void **);
    typedef int (*close_t)(void *);
    typedef const char *(*errmsg_t)(void *);
    typedef int (*exec_t)(void *, const char *, void *, void *, char **);
    auto s_open = (open_t)dlsym(h, "sqlite3_open");
    auto s_close = (close_t)dlsym(h, "sqlite3_close");
    auto s_errmsg = (errmsg_t)dlsym(h, "sqlite3_errmsg");
    auto s_exec = (exec_t)dlsym(h, "sqlite3_exec");
    if (!s_open || !s_close || !s_errmsg || !s_exec) return 1;
    void *db = nullptr;
    if (s_open(c.search_db.c_str(), &db) != 0) {
        printf("Can't open database(%s): %s\n", c.search_db.c_str(), s_errmsg(db));
        return 1;
    }
    char sql[400];
    snprintf(sql, sizeof sql,
             "INSERT INTO range(rid, P,D, m_start,m_inc,sieve_length, max_prime,min_merit,num_m,"
             "time_sieve)VALUES(%ld,  %d,%d, %ld,%ld,%d,%ld, %.3f,%ld,  %.2f)"
             "ON CONFLICT(rid) DO UPDATE SET time_sieve=%.2f",
             (long)config_hash(c), (int)c.p, (int)c.d, (long)c.mstart, (long)c.minc,
             (int)c.sieve_length, (long)c.max_prime, c.min_merit, num_rows, time_sieve, time_sieve);
    char *zerr = nullptr;
    int rc = s_exec(db, sql, nullptr, nullptr, &zerr);
    if (rc != 0) {
        printf("\nrange INSERT failed %d: %s\n", rc, s_errmsg(db));
        s_close(db);
        return 1;
    }
    s_close(db);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    Config c = argparse(argc, argv, show_usage);
    if (c.valid == 0) {
        show_usage(argv[0]);
        return 1;
    }
    // set_defaults (combined_sieve.cpp:160-344)
    if (c.d % 4 == 0) d_optimizer(c);
    if (c.sieve_length == 0) {
        c.sieve_length = auto_sieve_length(c);
        assert(c.sieve_length > 100);
    }
    if (c.max_prime == 0) {
        const double K_log = k_log(build_k(c.p, c.d));
        c.max_prime = K_log >= 1500 ? 100000000000ull : 10000000000ull;
        if (c.method1) {
            printf("Can't use method1 and not set max_prime");
            return 1;
        }
        if (c.verbose >= 0) {
            printf("AUTO SET: max_prime (log(K) = ~%.0f): %llu\n", K_log, (unsigned long long)c.max_prime);
            printf("WATCH for 'Estimated 2x faster (CTRL+C to stop sieving)' warning");
        }
    }
    // main()'s checks (combined_sieve.cpp:86-135)
    if (!c.save_unknowns && !c.testing) {
        printf("Must set --save-unknowns\n");
        return 1;
    }
    if (c.sieve_length < 6 * c.p || c.sieve_length > 22 * c.p) {
        int sl_min = ((c.p * 8 - 1) / 500 + 1) * 500;
        int sl_max = ((c.p * 20 - 1) / 500 + 1) * 500;
        printf("--sieve_length(%d) should be between [%d, %d]\n", c.sieve_length, sl_min, sl_max);
        return 1;
    }
    const std::string fn = gen_unknown_fn(c);
    if (c.save_unknowns && file_exists(fn)) {
        printf("\nOutput file '%s' already exists\n", fn.c_str());
        return 1;
    }
    if (!c.compression && (c.minc * c.sieve_length) > 100000000000ull) {
        printf("\tSetting --bitcompress to prevent very large output file\n");
        c.compression = 2;
    }
    if (!c.compression && (c.minc * c.sieve_length) > 30000000000ull) {
        printf("\tSetting --rle to prevent very large output file\n");
        c.compression = 1;
    }
    if (c.verbose >= 0) {
        printf("\n");
        printf("Testing m * %u#/%u, m = %llu + [0, %llu)\n", c.p, c.d, (unsigned long long)c.mstart,
               (unsigned long long)c.minc);
    }

    auto t0 = std::chrono::steady_clock::now();
    pgs_ctx *ctx = nullptr;
    int rc = pgs_create(0, &ctx);
    if (rc != PGS_OK) {
        printf("no CUDA device available (%d)\n", rc);
        return 1;
    }
    pgs_job job{c.p, c.d, c.mstart, c.minc, c.sieve_length, c.max_prime,
                c.compression == 3 ? 0 : c.compression, 0};
    pgs_result res;
    rc = c.method1 ? pgs_method1(ctx, &job, &res) : pgs_method2(ctx, &job, &res);
    if (rc != PGS_OK) {
        printf("combined_sieve failed (%d): %s\n", rc, pgs_last_error(ctx));
        pgs_destroy(ctx);
        return 1;
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (c.verbose >= 1) {
        printf("sieve_length:  2x %u\n", c.sieve_length);
        printf("max_prime:        %llu\n", (unsigned long long)c.max_prime);
        printf("primes sieved:    %llu\n", (unsigned long long)res.primes);
        printf("device time:      %.2f ms\n", res.ms_total);
    }
    int exit_code = 0;
    if (c.save_unknowns) {
        printf("\nSaving unknowns to '%s'\n", fn.c_str());
        FILE *f = fopen(fn.c_str(), "wb");
        if (!f) {
            printf("can't open '%s'\n", fn.c_str());
            exit_code = 1;
        } else {
            size_t w = fwrite(res.text, 1, res.text_len, f);
            if (fclose(f) != 0 || w != res.text_len) exit_code = 1;
        }
        if (!exit_code) exit_code = insert_range_db(c, (long)res.rows, (float)(c.threads * secs));
    }
    pgs_result_free(&res);
    pgs_destroy(ctx);
    return exit_code;
}
