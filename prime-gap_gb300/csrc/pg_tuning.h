// Tuning classes and the tuning cache file (host C++ only; also compiled into
// the CPU tests).
//
// A job's class is (P, floor(log2 SL), floor(log2 minc), floor(log2
// max_prime)): the knobs that the tuner picks depend on the prime phase's
// shape -- the continued fractions' depth and the walks' lengths (P's K, the
// window 2*SL+1, the walk length minc) and the primes' count and width
// (max_prime) -- more than on the exact values.  The cache file has one line per
// (device, class):
//   device <TAB> class <TAB> direct item_steps heavy rows chunks lsb form <TAB> ms_default ms_tuned
// Lines starting with '#' are comments.  Saving merges with the file's other
// devices' lines.
#pragma once
#include <stdint.h>

#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "pgsieve.h"

namespace pgt {

inline int ilog2(uint64_t v) {
    int b = -1;
    while (v) v >>= 1, b++;
    return b;
}

inline std::string tuning_class(const pgs_job &j) {
    std::ostringstream o;
    o << "P" << j.p << ".SL" << ilog2(j.sieve_length) << ".minc" << ilog2(j.minc) << ".mp" << ilog2(j.max_prime);
    return o.str();
}

inline pgs_tuning tuning_default() {
    pgs_tuning t;
    t.direct_steps = 24;
    t.item_steps = 64;
    t.heavy_steps = 4096;
    t.rows_per_cta = 16;
    t.text_chunks = 4;
    t.kmod_lsb_limbs = 32;
    t.large_form = 0;
    return t;
}

// Values inside the ranges the kernels accept.
inline bool tuning_valid(const pgs_tuning &t) {
    return t.direct_steps >= 1 && t.direct_steps <= 1024 &&
           (t.item_steps == 32 || t.item_steps == 64 || t.item_steps == 128) && t.heavy_steps >= 256 &&
           t.heavy_steps <= (1u << 24) && t.heavy_steps >= t.direct_steps && t.rows_per_cta >= 1 &&
           t.rows_per_cta <= 32 && t.text_chunks >= 1 && t.text_chunks <= 4 && t.kmod_lsb_limbs >= 1 &&
           t.large_form <= 7;
}

struct Entry {
    pgs_tuning t;
    double ms_default = 0, ms_tuned = 0;
};

inline std::string format_line(const std::string &device, const std::string &cls, const Entry &e) {
    std::ostringstream o;
    o << device << '\t' << cls << '\t' << e.t.direct_steps << ' ' << e.t.item_steps << ' ' << e.t.heavy_steps << ' '
      << e.t.rows_per_cta << ' ' << e.t.text_chunks << ' ' << e.t.kmod_lsb_limbs << ' ' << e.t.large_form << '\t'
      << e.ms_default << ' ' << e.ms_tuned;
    return o.str();
}

// false for comments, blank or malformed lines.
inline bool parse_line(const std::string &line, std::string &device, std::string &cls, Entry &e) {
    if (line.empty() || line[0] == '#') return false;
    std::vector<std::string> f;
    std::string cur;
    for (char c : line) {
        if (c == '\t') {
            f.push_back(cur);
            cur.clear();
        } else if (c != '\r' && c != '\n') {
            cur += c;
        }
    }
    f.push_back(cur);
    if (f.size() < 3 || f[0].empty() || f[1].empty()) return false;
    std::istringstream v(f[2]);
    if (!(v >> e.t.direct_steps >> e.t.item_steps >> e.t.heavy_steps >> e.t.rows_per_cta >> e.t.text_chunks >>
          e.t.kmod_lsb_limbs >> e.t.large_form))
        return false;
    if (!tuning_valid(e.t)) return false;
    e.ms_default = e.ms_tuned = 0;
    if (f.size() > 3) {
        std::istringstream m(f[3]);
        m >> e.ms_default >> e.ms_tuned;
    }
    device = f[0];
    cls = f[1];
    return true;
}

// Entries of `device` in the file (added to `m`); -1 when it cannot be read.
inline int load(const std::string &path, const std::string &device, std::map<std::string, Entry> &m) {
    std::ifstream in(path);
    if (!in) return -1;
    std::string line, dev, cls;
    int n = 0;
    while (std::getline(in, line)) {
        Entry e;
        if (parse_line(line, dev, cls, e) && dev == device) m[cls] = e, n++;
    }
    return n;
}

// The file's lines of other devices, then `device`'s entries; -1 on error.
inline int save(const std::string &path, const std::string &device, const std::map<std::string, Entry> &m) {
    std::vector<std::string> keep;
    {
        std::ifstream in(path);
        std::string line, dev, cls;
        while (in && std::getline(in, line)) {
            Entry e;
            if (parse_line(line, dev, cls, e) && dev != device) keep.push_back(line);
        }
    }
    std::ofstream out(path, std::ios::trunc);
    if (!out) return -1;
    out << "# libpgsieve tuning: device, class (P.SL<log2>.minc<log2>.mp<log2>), direct item_steps heavy rows chunks "
           "kmod_lsb large_form, ms default and tuned\n";
    for (const auto &l : keep) out << l << '\n';
    for (const auto &kv : m) out << format_line(device, kv.first, kv.second) << '\n';
    return out ? (int)m.size() : -1;
}

}  // namespace pgt
