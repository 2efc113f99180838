/*
 * Test infrastructure only: a stand-in for the primesieve library (absent on
 * the build host) with the subset of its documented interface the reference
 * uses.  A fresh iterator(start) yields the first prime >= start from
 * next_prime() and the first prime <= start from prev_prime(); later calls move
 * strictly up or down from the last prime returned.  Primes come from a
 * segmented sieve of Eratosthenes over buffered windows of the number line.
 */
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

namespace primesieve {

namespace detail {
// Odd primes below 2^21: enough to sieve any window below 2^42.
inline const std::vector<uint32_t> &seed_primes() {
    static const std::vector<uint32_t> primes = [] {
        const uint32_t limit = 1u << 21;
        std::vector<uint8_t> composite(limit, 0);
        std::vector<uint32_t> out;
        for (uint32_t i = 3; i < limit; i += 2) {
            if (composite[i]) continue;
            out.push_back(i);
            for (uint64_t j = (uint64_t)i * i; j < limit; j += 2 * i) composite[j] = 1;
        }
        return out;
    }();
    return primes;
}

// All primes in [lo, hi), ascending.
inline void primes_in_window(uint64_t lo, uint64_t hi, std::vector<uint64_t> &out) {
    out.clear();
    if (hi <= lo) return;
    if (lo <= 2 && 2 < hi) out.push_back(2);
    uint64_t first_odd = std::max<uint64_t>(lo, 3) | 1;
    if (first_odd >= hi) return;
    uint64_t count = (hi - first_odd + 1) / 2;  // odd numbers first_odd, first_odd+2, ...
    std::vector<uint8_t> dead(count, 0);
    for (uint32_t p : seed_primes()) {
        uint64_t sq = (uint64_t)p * p;
        if (sq >= hi) break;
        uint64_t start = std::max<uint64_t>(sq, (first_odd + p - 1) / p * p);
        if ((start & 1) == 0) start += p;
        for (uint64_t idx = (start - first_odd) / 2; idx < count; idx += p) dead[idx] = 1;
    }
    for (uint64_t i = 0; i < count; i++)
        if (!dead[i]) out.push_back(first_odd + 2 * i);
}
}  // namespace detail

class iterator {
  public:
    explicit iterator(uint64_t start = 0, uint64_t /*stop_hint*/ = 0) : start_(start) {
        detail::seed_primes();
    }

    uint64_t next_prime() {
        if (!started_) {
            started_ = true;
            fill_up(start_);
        } else if (idx_ + 1 >= (int64_t)buf_.size()) {
            fill_up(buf_.empty() ? start_ + 1 : buf_.back() + 1);
        } else {
            return buf_[++idx_];
        }
        idx_ = 0;
        return buf_[0];
    }

    uint64_t prev_prime() {
        if (!started_) {
            started_ = true;
            if (!fill_down(start_ + 1)) return 0;
        } else if (idx_ <= 0) {
            if (buf_.empty() || !fill_down(buf_.front())) return 0;
        } else {
            return buf_[--idx_];
        }
        idx_ = (int64_t)buf_.size() - 1;
        return buf_[idx_];
    }

  private:
    uint64_t start_;
    bool started_ = false;
    std::vector<uint64_t> buf_;
    int64_t idx_ = -1;
    uint64_t width_ = 1u << 15;

    void grow() {
        if (width_ < (1u << 21)) width_ <<= 1;
    }
    // Buffer the primes of the first non-empty window at or above `from`.
    void fill_up(uint64_t from) {
        while (true) {
            detail::primes_in_window(from, from + width_, buf_);
            from += width_;
            grow();
            if (!buf_.empty()) return;
        }
    }
    // Buffer the primes of the first non-empty window below `to`.
    bool fill_down(uint64_t to) {
        while (to > 2) {
            uint64_t lo = to > width_ ? to - width_ : 0;
            detail::primes_in_window(lo, to, buf_);
            grow();
            if (!buf_.empty()) return true;
            to = lo;
        }
        buf_.clear();
        return false;
    }
};

template <typename T>
void generate_primes(uint64_t stop, std::vector<T> *out) {
    std::vector<uint64_t> window;
    detail::primes_in_window(0, stop + 1, window);
    for (uint64_t p : window) out->push_back((T)p);
}

}  // namespace primesieve
