// Shared by the drop-in command-line tools (combined_sieve, gap_test): the
// reference's Config fields and Args::argparse (gap_common.h:39-89,
// gap_common.cpp:805-1099), its unknowns file name (Args::gen_unknown_fn,
// gap_common.cpp:732-749) and K = p#/d helpers (gap_common.cpp:100-121).
#pragma once
#include <getopt.h>
#include <libgen.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace pgcli {

struct Config {
    int valid = 1;
    uint32_t p = 0, d = 0;
    uint64_t mstart = 0, minc = 0, mskip = 0;
    float min_merit = 18;
    uint32_t sieve_length = 0;
    uint64_t max_prime = 0;
    bool save_unknowns = false, method1 = false, show_timing = true, testing = false;
    int compression = 0, threads = 1, max_mem = 10, verbose = 2;
    std::string unknown_filename;
    std::string search_db = "prime-gap-search.db";
    std::string gaps_db = "gaps.db";
};

inline bool file_exists(const std::string &path) {
    std::ifstream f(path);
    return f.good();
}

inline void require_file(const char *path) {
    if (!file_exists(path)) {
        printf("'%s' doesn't exist\n", path);
        exit(1);
    }
}

inline bool is_prime_brute(uint64_t n) {
    if (n < 2) return false;
    if (n % 2 == 0) return n == 2;
    for (uint64_t t = 3; t * t <= n; t += 2)
        if (n % t == 0) return false;
    return true;
}

// ---- set_defaults (combined_sieve.cpp:160-344) and its helpers ----

inline uint64_t gcd_u64(uint64_t a, uint64_t b) { return b == 0 ? a : gcd_u64(b, a % b); }

inline std::vector<uint32_t> primes_upto(uint32_t n) {
    std::vector<uint32_t> out;
    std::vector<char> comp(n + 1, 0);
    for (uint32_t i = 2; i <= n; i++) {
        if (comp[i]) continue;
        out.push_back(i);
        for (uint64_t j = (uint64_t)i * i; j <= n; j += i) comp[j] = 1;
    }
    return out;
}

// K = p#/d as 32-bit limbs (init_K, gap_common.cpp:116-121; d divides p#)
inline std::vector<uint32_t> build_k(uint32_t p, uint32_t d) {
    std::vector<uint32_t> k{1};
    uint32_t rest = d;
    for (uint32_t q : primes_upto(p)) {
        if (rest % q == 0) {
            rest /= q;
            continue;
        }
        uint64_t c = 0;
        for (auto &l : k) {
            const uint64_t t = (uint64_t)l * q + c;
            l = (uint32_t)t;
            c = t >> 32;
        }
        if (c) k.push_back((uint32_t)c);
    }
    assert(rest == 1);
    return k;
}

inline uint32_t k_mod(const std::vector<uint32_t> &k, uint32_t d) {
    uint64_t r = 0;
    for (size_t i = k.size(); i-- > 0;) r = ((r << 32) | k[i]) % d;
    return (uint32_t)r;
}

// _log(K) (gap_common.cpp:100-104): GMP's truncated 53-bit mantissa in
// [0.5, 1) and its exponent
inline double k_log(const std::vector<uint32_t> &k) {
    const uint32_t b = 32u * (uint32_t)(k.size() - 1) + (32u - (uint32_t)__builtin_clz(k.back()));
    uint64_t top = 0;
    for (uint32_t i = 0; i < 53; i++) {
        const uint32_t bit = b >= i + 1 ? (k[(b - 1 - i) >> 5] >> ((b - 1 - i) & 31)) & 1u : 0u;
        top = (top << 1) | bit;
    }
    return std::log((double)top / 9007199254740992.0) + std::log(2.0) * b;
}

inline std::string gen_unknown_fn(const Config &c) {
    if (!c.unknown_filename.empty()) return c.unknown_filename;
    return "unknowns/" + std::to_string(c.p) + "_" + std::to_string(c.d) + "_" +
           std::to_string(c.mstart) + "_" + std::to_string(c.minc) + "_s" +
           std::to_string(c.sieve_length) + "_l" + std::to_string(c.max_prime / 1000000) + "M" +
           (c.method1 ? ".m1" : "") + ".txt";
}

inline Config argparse(int argc, char **argv, void (*usage)(const char *)) {
    static struct option long_options[] = {
        {"p", required_argument, 0, 'p'},
        {"d", required_argument, 0, 'd'},
        {"mstart", required_argument, 0, 1},
        {"minc", required_argument, 0, 2},
        {"mskip", required_argument, 0, 16},
        {"unknown-filename", required_argument, 0, 'u'},
        {"sieve-length", required_argument, 0, 4},
        {"max-prime", required_argument, 0, 5},
        {"threads", required_argument, 0, 't'},
        {"min-merit", required_argument, 0, 3},
        {"save", no_argument, 0, 7},
        {"save-unknowns", no_argument, 0, 7},
        {"rle", no_argument, 0, 13},
        {"bitcompressed", no_argument, 0, 15},
        {"uncompressed", no_argument, 0, 17},
        {"max-mem", required_argument, 0, 14},
        {"search-db", required_argument, 0, 9},
        {"prime-gaps-db", required_argument, 0, 10},
        {"method1", no_argument, 0, 8},
        {"hide-timing", no_argument, 0, 11},
        {"testing", no_argument, 0, 12},
        {"quiet", no_argument, 0, 'q'},
        {"help", no_argument, 0, 'h'},
        {0, 0, 0, 0}};
    Config c;
    int option_index = 0;
    int ch;
    while ((ch = getopt_long(argc, argv, "qhp:d:u:t:", long_options, &option_index)) >= 0) {
        switch (ch) {
            case 'h': usage(argv[0]); exit(0);
            case 'q': c.verbose--; break;
            case 'p': c.p = atoi(optarg); break;
            case 'd': c.d = atoi(optarg); break;
            case 1: c.mstart = atoll(optarg); break;
            case 2: c.minc = atoll(optarg); break;
            case 16: c.mskip = atoll(optarg); break;
            case 'u': {
                // <dir>/<P>_<d>_<mstart>_<minc>_s<SL>_l<MP>M[.m1].txt (gap_common.cpp:877-925)
                std::string full = optarg;
                char *t1 = strdup(optarg);
                std::string dir = dirname(t1);
                free(t1);
                char *t2 = strdup(optarg);
                std::string base = basename(t2);
                free(t2);
                dir = (dir == ".") ? "unknowns" : dir;
                c.unknown_filename = dir + "/" + base;
                unsigned us = 0;
                for (char x : base) us += x == '_';
                unsigned long long ms = 0, mi = 0, mp = 0;
                unsigned p = 0, d = 0, sl = 0;
                char tail[32] = {0};
                if (us != 5 || sscanf(base.c_str(), "%u_%u_%llu_%llu_s%u_l%llu%31s", &p, &d, &ms,
                                      &mi, &sl, &mp, tail) != 7 ||
                    (strcmp(tail, "M.txt") != 0 && strcmp(tail, "M.m1.txt") != 0)) {
                    printf("can't parse unknown filename '%s'\n", base.c_str());
                    exit(1);
                }
                c.p = p;
                c.d = d;
                c.mstart = ms;
                c.minc = mi;
                c.sieve_length = sl;
                c.max_prime = mp * 1000000ull;
                c.method1 = strcmp(tail, "M.m1.txt") == 0;
                break;
            }
            case 't': c.threads = atoi(optarg); break;
            case 3: c.min_merit = atof(optarg); break;
            case 4: c.sieve_length = atoi(optarg); break;
            case 5: c.max_prime = atol(optarg) * 1000000ull; break;
            case 7: c.save_unknowns = true; break;
            case 8: c.method1 = true; break;
            case 9: c.search_db = optarg; require_file(optarg); break;
            case 10: c.gaps_db = optarg; require_file(optarg); break;
            case 11: c.show_timing = false; break;
            case 12: c.testing = true; break;
            case 13: c.compression = 1; break;
            case 15: c.compression = 2; break;
            case 17: c.compression = 3; break;
            case 14: c.max_mem = atol(optarg); break;
            default: c.valid = 0;
        }
    }
    if (optind < argc) {
        c.valid = 0;
        printf("unknown positional argument: ");
        while (optind < argc) printf("%s ", argv[optind++]);
        printf("\n");
    }
    if (c.testing) c.save_unknowns = false;
    // validation (gap_common.cpp:1007-1094)
    if (c.mstart <= 0) {
        c.valid = 0;
        printf("mstart must be greater than 0: %llu\n", (unsigned long long)c.mstart);
    }
    int64_t last_m = (int64_t)(c.mstart + c.minc);
    if (last_m <= 0 || last_m > 10000000001LL) {
        c.valid = 0;
        printf("mstart + minc must be <= 10e9\n");
    }
    if (c.minc <= 0) {
        c.valid = 0;
        printf("minc must be greater than 0: %llu\n", (unsigned long long)c.minc);
    }
    if (c.minc >= 0x7FFFFFFFull) {
        c.valid = 0;
        printf("minc must be less than 2B %llu\n", (unsigned long long)c.minc);
    }
    if (c.max_prime > 40000000000000ull) {
        c.valid = 0;
        printf("max_prime > 40 Trillion not supported\n");
    }
    if (c.method1 && c.max_prime) {
        uint64_t max_m = UINT64_MAX / c.max_prime;
        if (max_m < 1000 || (max_m + 1000) <= (uint64_t)last_m) {
            c.valid = 0;
            printf("max_prime * last_m(%lld) would overflow int64\n", (long long)last_m);
        }
    }
    if (!(c.p < 10000000u && (c.p < 4 || is_prime_brute(c.p)))) {
        printf("p# not prime (p=%u)\n", c.p);
        exit(1);
    }
    if (c.sieve_length % 500 != 0) {
        for (uint32_t q = 2; q < c.p; q += 1 + (q > 2)) {
            if (is_prime_brute(q) && c.sieve_length % q == 0 && c.d % q != 0) {
                c.valid = 0;
                printf("SL=%u not coprime (p=%u)\n", c.sieve_length, q);
            }
        }
    }
    if (c.d <= 0) {
        c.valid = 0;
        printf("d must be greater than 0: %u\n", c.d);
    }
    if (c.threads <= 0 || c.threads > 16) {
        c.valid = 0;
        printf("invalid number of threads(%d) only 1 - 16 supported\n", c.threads);
    }
    if (c.valid == 0) printf("\n");
    return c;
}

}  // namespace pgcli
