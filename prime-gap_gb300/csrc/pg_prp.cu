// Probable-prime tests of N = m*K +- X on the device, and the prime-gap search
// over a job's unknown lists that they serve.
//
// Replaces the reference's GPU Miller-Rabin (kernel_miller_rabin,
// miller_rabin_t::miller_rabin and powm, miller_rabin.h:154-267: CGBN, eight
// threads per number) with the one base gap_test_gpu uses (ROUNDS = 1 with
// primes {2}, gap_test_gpu.cu:81, miller_rabin.h:269), and its host threads
// (load_batch_thread, run_gpu_thread, run_overflow_thread,
// gap_test_gpu.cu:213-640) with device rounds.
//
// Numbers: n = 8L little-endian 32-bit limbs over a group of 8 lanes of a
// warp, lane t holding limbs [tL, tL + L).  N < 2^(32n - 4), so R = 2^(32n) is
// at least 16N and Montgomery products of inputs below 4N stay below 2N: 2^d
// (N - 1 = d 2^s) by left-to-right squaring with a doubling (a one-bit shift)
// on each set bit of d needs no conditional subtraction.  Base 2 makes every
// multiplication of the exponentiation a shift.
//
// Montgomery product, CIOS word by word: each lane runs its L-limb
// multiply-add chains; the carry out of its top limb waits in a pending word
// until the one-limb shift of the step brings the next lane's bottom limb down
// beside it, so a step exchanges three words between lanes (the multiplier
// word, the quotient word, the shifted limb) and no carry crosses lanes until
// the end of the product, where one ballot resolves them all.
//
// The strong test follows miller_rabin.h:211-245, including its loop bound:
// after x = 2^d, up to s squarings (one more than the textbook s - 1).  The
// extra squaring never changes a verdict (2^(N-1) = -1 mod N has no odd
// solution N > 1).
#include <cmath>
#include <cstring>
#include <vector>

#include "pg_arith.cuh"
#include "pg_host.h"

namespace pg {

namespace {

constexpr int kTPI = 8;                       // lanes per number
constexpr int kPrpThreads = 128;              // 16 numbers per block
constexpr int kGroups = kPrpThreads / kTPI;
constexpr int kMaxL = 16;                     // up to 8*16*32 - 4 = 4092-bit numbers

template <int L>
struct Num {
    uint32_t v[L];
};

struct Grp {
    uint32_t mask;  // the group's lanes in the warp
    uint32_t base;  // its first lane
    uint32_t t;     // this lane within the group
};

__device__ __forceinline__ Grp group_of_lane() {
    const uint32_t lane = threadIdx.x & 31u;
    Grp g;
    g.t = lane & (kTPI - 1);
    g.base = lane - g.t;
    g.mask = ((1u << kTPI) - 1u) << g.base;
    return g;
}

__device__ __forceinline__ uint32_t gballot(const Grp &g, bool p) {
    return (__ballot_sync(g.mask, p) >> g.base) & ((1u << kTPI) - 1u);
}

// Carries between lanes from each lane's carry out (gen) and whether it would
// pass an incoming carry on (prop): bit t = carry into lane t, bit kTPI =
// carry out of the top lane.  Same rule for borrows.
__device__ __forceinline__ uint32_t lane_carries(uint32_t gen, uint32_t prop) {
    return ((gen << 1) + prop) ^ prop;
}

template <int L>
__device__ __forceinline__ uint32_t add_lane(Num<L> &a, uint32_t c) {
#pragma unroll
    for (int k = 0; k < L; k++) {
        const uint64_t s = (uint64_t)a.v[k] + c;
        a.v[k] = (uint32_t)s;
        c = (uint32_t)(s >> 32);
    }
    return c;
}

template <int L>
__device__ __forceinline__ uint32_t sub_lane(Num<L> &a, uint32_t b) {
#pragma unroll
    for (int k = 0; k < L; k++) {
        const uint64_t s = (uint64_t)a.v[k] - b;
        a.v[k] = (uint32_t)s;
        b = (uint32_t)(s >> 63);
    }
    return b;
}

template <int L>
__device__ __forceinline__ bool all_limbs(const Num<L> &a, uint32_t w) {
    bool r = true;
#pragma unroll
    for (int k = 0; k < L; k++) r &= a.v[k] == w;
    return r;
}

// a += x, x at limb 0
template <int L>
__device__ __forceinline__ void add_small(const Grp &g, Num<L> &a, uint32_t x) {
    const uint32_t co = add_lane(a, g.t == 0 ? x : 0u);
    const uint32_t cin = lane_carries(gballot(g, co != 0), gballot(g, all_limbs(a, 0xFFFFFFFFu)));
    add_lane(a, (cin >> g.t) & 1u);
}

// a -= x, x at limb 0, a >= x
template <int L>
__device__ __forceinline__ void sub_small(const Grp &g, Num<L> &a, uint32_t x) {
    const uint32_t bo = sub_lane(a, g.t == 0 ? x : 0u);
    const uint32_t bin = lane_carries(gballot(g, bo != 0), gballot(g, all_limbs(a, 0u)));
    sub_lane(a, (bin >> g.t) & 1u);
}

// a -= n when a >= n (a < 2n)
template <int L>
__device__ __forceinline__ void reduce_once(const Grp &g, Num<L> &a, const Num<L> &n) {
    Num<L> d;
    uint32_t br = 0;
#pragma unroll
    for (int k = 0; k < L; k++) {
        const uint64_t s = (uint64_t)a.v[k] - n.v[k] - br;
        d.v[k] = (uint32_t)s;
        br = (uint32_t)(s >> 63);
    }
    const uint32_t bin = lane_carries(gballot(g, br != 0), gballot(g, all_limbs(d, 0u)));
    sub_lane(d, (bin >> g.t) & 1u);
    if (!((bin >> kTPI) & 1u)) a = d;  // no borrow out of the top: a >= n
}

// a <<= bit (bit 0 or 1)
template <int L>
__device__ __forceinline__ void shl(const Grp &g, Num<L> &a, uint32_t bit) {
    uint32_t in = __shfl_up_sync(g.mask, a.v[L - 1], 1, kTPI);
    if (g.t == 0) in = 0;
#pragma unroll
    for (int k = L - 1; k > 0; k--) a.v[k] = __funnelshift_l(a.v[k - 1], a.v[k], bit);
    a.v[0] = __funnelshift_l(in, a.v[0], bit);
}

// out = x * y / R mod n (below 2n for x, y below 4n), y = x or one (y_one).
template <int L>
__device__ __forceinline__ void mont_mul(const Grp &g, Num<L> &out, const Num<L> &x, bool y_one,
                                         const Num<L> &n, uint32_t ninv) {
    Num<L> y, a;
#pragma unroll
    for (int k = 0; k < L; k++) {
        y.v[k] = y_one ? (g.t == 0 && k == 0 ? 1u : 0u) : x.v[k];
        a.v[k] = 0;
    }
    uint64_t e = 0;  // carries pending into the next lane's bottom limb
    const bool top = g.t == kTPI - 1;
    for (uint32_t src = 0; src < kTPI; src++) {
#pragma unroll
        for (int k = 0; k < L; k++) {
            const uint32_t xi = __shfl_sync(g.mask, x.v[k], src, kTPI);
            uint32_t c = 0;
#pragma unroll
            for (int j = 0; j < L; j++) {
                const uint64_t s = (uint64_t)xi * y.v[j] + a.v[j] + c;
                a.v[j] = (uint32_t)s;
                c = (uint32_t)(s >> 32);
            }
            e += c;
            // lane 0's bottom limb has nothing pending: the quotient word
            const uint32_t q = __shfl_sync(g.mask, a.v[0] * ninv, 0, kTPI);
            c = 0;
#pragma unroll
            for (int j = 0; j < L; j++) {
                const uint64_t s = (uint64_t)q * n.v[j] + a.v[j] + c;
                a.v[j] = (uint32_t)s;
                c = (uint32_t)(s >> 32);
            }
            e += c;
            // shift down one limb; lane 0's bottom limb (zero) drops out
            uint32_t in = __shfl_down_sync(g.mask, a.v[0], 1, kTPI);
            if (top) in = 0;
#pragma unroll
            for (int j = 0; j + 1 < L; j++) a.v[j] = a.v[j + 1];
            const uint64_t s = (uint64_t)in + e;
            a.v[L - 1] = (uint32_t)s;
            e = s >> 32;
        }
    }
    // resolve the pending carries (the value is below R: none leaves the top)
    uint32_t in = __shfl_up_sync(g.mask, (uint32_t)e, 1, kTPI);
    if (g.t == 0) in = 0;
    const uint32_t co = add_lane(a, in);
    const uint32_t cin = lane_carries(gballot(g, co != 0), gballot(g, all_limbs(a, 0xFFFFFFFFu)));
    add_lane(a, (cin >> g.t) & 1u);
    out = a;
}

template <int L>
__device__ __forceinline__ bool equals_small(const Grp &g, const Num<L> &a, uint32_t w) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < L; k++) ok &= a.v[k] == (g.t == 0 && k == 0 ? w : 0u);
    return gballot(g, ok) == (1u << kTPI) - 1u;
}

template <int L>
__device__ __forceinline__ bool equals_n_minus_1(const Grp &g, const Num<L> &a, const Num<L> &n) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < L; k++) ok &= a.v[k] == n.v[k] - (g.t == 0 && k == 0 ? 1u : 0u);
    return gballot(g, ok) == (1u << kTPI) - 1u;
}

template <int L>
__device__ __forceinline__ uint32_t bit_length(const Grp &g, const Num<L> &a) {
    int hi = -1;
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < L; k++)
        if (a.v[k]) hi = k, w = a.v[k];
    const uint32_t lanes = gballot(g, hi >= 0);
    if (!lanes) return 0;
    const uint32_t top = 31 - __clz(lanes);
    const uint32_t word = __shfl_sync(g.mask, w, top, kTPI);
    const int idx = __shfl_sync(g.mask, hi, top, kTPI);
    return 32u * (top * L + (uint32_t)idx) + (32u - __clz(word));
}

// Base-2 strong probable-prime test of odd n (5 <= n < 2^(32*8L - 4)); sn =
// the group's copy of n's limbs in shared memory (exponent bits).
template <int L>
__device__ bool prp2(const Grp &g, const Num<L> &n, const uint32_t *sn) {
    const uint32_t b = bit_length(g, n);
    uint32_t s = 0;  // trailing zeros of n - 1
    for (uint32_t w = 0; w < 8u * L; w++) {
        const uint32_t v = sn[w] - (w == 0 ? 1u : 0u);
        if (v) {
            s = 32u * w + (uint32_t)__ffs(v) - 1u;
            break;
        }
    }
    const uint32_t ninv = __shfl_sync(g.mask, neg_inv32(n.v[0]), 0, kTPI);
    // x = 2R mod n, the Montgomery form of 2 (the leading bit of d): 2^(b-1)
    // doubled 32n - b + 2 times, reduced after each doubling
    Num<L> x;
    const uint32_t top_limb = (b - 1) >> 5;
#pragma unroll
    for (int k = 0; k < L; k++) x.v[k] = (g.t * L + k == top_limb) ? (1u << ((b - 1) & 31)) : 0u;
    const uint32_t doublings = 32u * 8u * L - b + 2u;
    for (uint32_t i = 0; i < doublings; i++) {
        shl(g, x, 1u);
        reduce_once(g, x, n);
    }
    // One Montgomery product per step: squarings of the exponent (bits b-2 ..
    // s of n are the bits of d below its leading one), then alternately a
    // conversion y = x/R (the value) and a squaring, per miller_rabin.h:222-243.
    int p = (int)b - 2;
    bool convert = p < (int)s;
    bool first_check = true;
    uint32_t count = s;
    for (;;) {
        Num<L> r;
        mont_mul(g, r, x, convert, n, ninv);
        if (!convert) {
            x = r;
            if (p >= (int)s) {
                const uint32_t bit = (sn[p >> 5] >> (p & 31)) & 1u;
                shl(g, x, bit);
                p--;
                convert = p < (int)s;
            } else {
                convert = true;  // a squaring of the strong loop: check it next
            }
            continue;
        }
        reduce_once(g, r, n);  // the value, below n
        convert = false;
        if (first_check) {
            if (equals_small(g, r, 1u) || equals_n_minus_1(g, r, n)) return true;
            if (s == 1) return false;
            first_check = false;
            continue;
        }
        if (equals_n_minus_1(g, r, n)) return true;
        if (--count == 0 || equals_small(g, r, 1u)) return false;
    }
}

struct PrpItem {
    uint32_t row;  // row of the base numbers
    int32_t x;     // N = base[row] + x
};

template <int L>
__global__ void __launch_bounds__(kPrpThreads)
    prp_kernel(const uint32_t *__restrict__ bases, const PrpItem *__restrict__ items,
               const unsigned long long *count, uint64_t max_items, uint8_t *__restrict__ result) {
    __shared__ uint32_t s_n[kGroups][8 * L];
    const Grp g = group_of_lane();
    const uint32_t gi = threadIdx.x / kTPI;
    const uint64_t i = (uint64_t)blockIdx.x * kGroups + gi;
    const uint64_t n_items = count ? min((uint64_t)*count, max_items) : max_items;
    if (i >= n_items) return;  // the whole group leaves together
    const PrpItem it = items[i];
    const uint32_t *src = bases + (uint64_t)it.row * (8 * L) + g.t * L;
    Num<L> n;
#pragma unroll
    for (int k = 0; k < L; k++) n.v[k] = src[k];
    if (it.x > 0) add_small(g, n, (uint32_t)it.x);
    if (it.x < 0) sub_small(g, n, (uint32_t)(-(int64_t)it.x));
#pragma unroll
    for (int k = 0; k < L; k++) s_n[gi][g.t * L + k] = n.v[k];
    __syncwarp(g.mask);
    const bool r = prp2<L>(g, n, s_n[gi]);
    if (g.t == 0) result[i] = r ? 1 : 0;
}

cudaError_t launch_prp(int L, const uint32_t *bases, const PrpItem *items, const unsigned long long *count,
                       uint64_t max_items, uint8_t *result, cudaStream_t s) {
    if (max_items == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((max_items + kGroups - 1) / kGroups);
#define PG_PRP_CASE(LL)                                                                               \
    case LL:                                                                                          \
        prp_kernel<LL><<<blocks, kPrpThreads, 0, s>>>(bases, items, count, max_items, result);        \
        break;
    switch (L) {
        PG_PRP_CASE(1)
        PG_PRP_CASE(2)
        PG_PRP_CASE(3)
        PG_PRP_CASE(4)
        PG_PRP_CASE(5)
        PG_PRP_CASE(6)
        PG_PRP_CASE(7)
        PG_PRP_CASE(8)
        PG_PRP_CASE(9)
        PG_PRP_CASE(10)
        PG_PRP_CASE(11)
        PG_PRP_CASE(12)
        PG_PRP_CASE(13)
        PG_PRP_CASE(14)
        PG_PRP_CASE(15)
        PG_PRP_CASE(16)
        default:
            return cudaErrorInvalidValue;
    }
#undef PG_PRP_CASE
    return cudaGetLastError();
}

// Limbs per lane for numbers of `bits` bits: 32*8L >= bits + 4.
int limbs_per_lane(uint32_t bits) { return (int)((bits + 4 + 255) / 256); }

// ---------------------------------------------------------------------------
// gap search

// centers[r] = m[r] * K as n limbs (one thread per row)
__global__ void centers_kernel(const uint32_t *__restrict__ k, uint32_t nk, const uint64_t *__restrict__ m,
                               uint64_t rows, uint32_t n, uint32_t *__restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const uint64_t mm = m[r];
    const uint32_t lo = (uint32_t)mm, hi = (uint32_t)(mm >> 32);
    uint32_t *o = out + r * n;
    uint64_t c = 0;
    for (uint32_t j = 0; j < n; j++) {
        const uint64_t t = (uint64_t)lo * (j < nk ? k[j] : 0u) + c;
        o[j] = (uint32_t)t;
        c = t >> 32;
    }
    c = 0;
    for (uint32_t j = 1; j < n; j++) {
        const uint64_t t = (uint64_t)hi * (j - 1 < nk ? k[j - 1] : 0u) + o[j] + c;
        o[j] = (uint32_t)t;
        c = t >> 32;
    }
}

struct GapRow {
    uint32_t side;        // 0: previous prime, 1: next prime, 2: done
    uint32_t idx;         // next unknown to test on this side
    uint32_t past;        // 1 while this side searches past the sieve length
    uint32_t past_x;      // next distance to scan past the sieve length
    uint32_t item_base, item_cnt;
    uint32_t skip_below;  // next side skipped when prev_p < skip_below (0: never)
    uint32_t center_odd;  // parity of m*K
};

struct GapLists {
    const uint64_t *start;
    const uint32_t *n_prev, *n_next, *dist;
};

__device__ __forceinline__ bool coprime_to_k(uint32_t x, const uint32_t *kp, uint32_t nkp) {
    for (uint32_t i = 0; i < nkp; i++)
        if (x % kp[i] == 0) return false;
    return true;
}

// Candidates of this round: up to spec per active row, nearest first; past
// the sieve length, the next spec distances that keep N odd and coprime to K.
__global__ void select_kernel(GapRow *rows_st, uint64_t rows, GapLists ls, uint32_t spec, const uint32_t *kp,
                              uint32_t nkp, uint32_t x_limit, PrpItem *items, uint64_t max_items,
                              unsigned long long *n_items, unsigned long long *errors) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    GapRow st = rows_st[r];
    st.item_cnt = 0;
    if (st.side < 2) {
        const int32_t sign = st.side == 0 ? -1 : 1;
        if (!st.past) {
            const uint32_t nlist = st.side == 0 ? ls.n_prev[r] : ls.n_next[r];
            const uint32_t *lst = ls.dist + ls.start[r] + (st.side == 0 ? 0u : ls.n_prev[r]);
            uint32_t cnt = min(spec, nlist - st.idx);
            const uint64_t base = atomicAdd(n_items, (unsigned long long)cnt);
            if (base + cnt > max_items) {  // the host sizes rounds so that this never happens
                atomicAdd(errors, 1ull);
                st.side = 2;
                cnt = 0;
            }
            for (uint32_t j = 0; j < cnt; j++) items[base + j] = PrpItem{(uint32_t)r, sign * (int32_t)lst[st.idx + j]};
            st.item_base = (uint32_t)base;
            st.item_cnt = cnt;
        } else {
            const uint64_t base = atomicAdd(n_items, (unsigned long long)spec);
            uint32_t x = st.past_x, cnt = 0;
            if (base + spec > max_items) {
                atomicAdd(errors, 1ull);
                st.side = 2;
                rows_st[r] = st;
                return;
            }
            // N = m*K +- x odd: x of the other parity than m*K
            if ((x & 1u) == st.center_odd) x++;
            while (cnt < spec && x < x_limit) {
                if (coprime_to_k(x, kp, nkp)) items[base + cnt++] = PrpItem{(uint32_t)r, sign * (int32_t)x};
                x += 2;
            }
            if (cnt < spec) {
                atomicAdd(errors, 1ull);  // no prime within the scan limit: report, stop the row
                st.side = 2;
                // the reserved slots left over get a harmless item (N = m*K)
                for (uint32_t j = cnt; j < spec; j++) items[base + j] = PrpItem{(uint32_t)r, 0};
            }
            st.item_base = (uint32_t)base;
            st.item_cnt = cnt;
            st.past_x = x;
        }
    }
    rows_st[r] = st;
}

__global__ void resolve_kernel(GapRow *rows_st, uint64_t rows, GapLists ls, const PrpItem *items,
                               const uint8_t *result, uint32_t sl, pgs_gap_result *out,
                               unsigned long long *active) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    GapRow st = rows_st[r];
    if (st.side >= 2 || st.item_cnt == 0) return;
    int first = -1;
    for (uint32_t j = 0; j < st.item_cnt; j++)
        if (result[st.item_base + j]) {
            first = (int)j;
            break;
        }
    pgs_gap_result o = out[r];
    const uint32_t nlist = st.side == 0 ? ls.n_prev[r] : ls.n_next[r];
    if (first < 0) {
        if (!st.past) {
            st.idx += st.item_cnt;
            if (st.idx >= nlist) st.past = 1, st.past_x = sl + 1;
        }
    } else {
        const int32_t xs = items[st.item_base + first].x;
        const uint32_t x = (uint32_t)(xs < 0 ? -xs : xs);
        const uint32_t tests = st.past ? nlist : st.idx + (uint32_t)first + 1u;
        if (st.side == 0) {
            o.prev_p = (int32_t)x;
            o.p_tests = tests;
            o.flags |= st.past ? 1u : 0u;
            if (x < st.skip_below) {
                st.side = 2;
                o.flags |= 4u;
            } else {
                st.side = 1;
                st.idx = 0;
                st.past = ls.n_next[r] == 0 ? 1u : 0u;
                st.past_x = sl + 1;
            }
        } else {
            o.next_p = (int32_t)x;
            o.n_tests = tests;
            o.flags |= st.past ? 2u : 0u;
            st.side = 2;
        }
        out[r] = o;
    }
    rows_st[r] = st;
    if (st.side < 2) atomicAdd(active, 1ull);
}

__global__ void gap_init_kernel(GapRow *rows_st, uint64_t rows, GapLists ls, const uint32_t *skip_below,
                                const uint32_t *centers, uint32_t n, uint32_t sl, pgs_gap_result *out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    GapRow st{};
    st.side = 0;
    st.past = ls.n_prev[r] == 0 ? 1u : 0u;
    st.past_x = sl + 1;
    st.skip_below = skip_below ? skip_below[r] : 0u;
    st.center_odd = centers[r * n] & 1u;
    rows_st[r] = st;
    out[r] = pgs_gap_result{};
}

}  // namespace

}  // namespace pg

using namespace pgh;

namespace {

// K = p#/d as 32-bit limbs (gap_common.cpp:116-121).
bool build_k(uint32_t p, uint32_t d, std::vector<uint32_t> &k, std::vector<uint32_t> &k_primes) {
    k.assign(1, 1u);
    uint32_t rest = d;
    for (uint32_t q : primes_upto(p)) {
        if (rest % q == 0) {
            rest /= q;
            continue;
        }
        k_primes.push_back(q);
        uint64_t c = 0;
        for (auto &l : k) {
            const uint64_t t = (uint64_t)l * q + c;
            l = (uint32_t)t;
            c = t >> 32;
        }
        if (c) k.push_back((uint32_t)c);
    }
    return rest == 1;
}

uint32_t bits_of(const std::vector<uint32_t> &k) {
    return 32u * (uint32_t)(k.size() - 1) + (32u - (uint32_t)__builtin_clz(k.back()));
}

// _log(K) (gap_common.cpp:100-104): log of GMP's truncated 53-bit mantissa in
// [0.5, 1) plus exp * log(2).
double k_log(const std::vector<uint32_t> &k) {
    const uint32_t b = bits_of(k);
    auto bit = [&](uint32_t i) { return (k[i >> 5] >> (i & 31)) & 1u; };
    uint64_t top = 0;
    for (uint32_t i = 0; i < 53; i++) top = (top << 1) | (b >= 1 + i ? bit(b - 1 - i) : 0u);
    const double mantissa = (double)top / 9007199254740992.0;  // 2^53
    return std::log(mantissa) + std::log(2.0) * b;
}

// Smallest prev_p whose merit, float(prev_p / (K_log + log(m))), reaches
// min_merit / 2 - 2 (gap_test_gpu.cu:577-590); 0 when every prev_p does.
uint32_t skip_threshold(double klog, uint64_t m, float min_merit) {
    const float need = min_merit / 2 - 2;
    const double denom = klog + std::log((double)m);
    auto ok = [&](uint32_t g) { return !((float)(g / denom) < need); };
    if (ok(0)) return 0;
    uint32_t lo = 0, hi = 1;
    while (!ok(hi)) {
        lo = hi;
        if (hi >= 0x40000000u) return 0x7FFFFFFFu;
        hi *= 2;
    }
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        (ok(mid) ? hi : lo) = mid;
    }
    return hi;
}

constexpr uint64_t kRoundTarget = 1ull << 15;  // candidates per round when few rows remain
constexpr uint32_t kMaxSpec = 64;
constexpr uint32_t kPastScanSpan = 1u << 24;   // distances scanned past SL before giving up

}  // namespace

extern "C" {

int pgs_prp_test(pgs_ctx *ctx, const uint32_t *limbs, uint32_t n_limbs, size_t count, int rounds,
                 uint8_t *out) {
    if (!ctx || (count && (!limbs || !out)) || n_limbs == 0 || rounds != 1) return PGS_EINVAL;
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    if (count == 0) return PGS_OK;
    // width from the largest number; tiny, even and too wide numbers on the host
    uint32_t max_bits = 0;
    std::vector<uint64_t> dev_rows;
    for (size_t i = 0; i < count; i++) {
        const uint32_t *v = limbs + i * n_limbs;
        uint32_t top = n_limbs;
        while (top > 0 && v[top - 1] == 0) top--;
        const uint32_t bits = top ? 32u * (top - 1) + (32u - (uint32_t)__builtin_clz(v[top - 1])) : 0u;
        if (bits > 8u * pg::kMaxL * 32u - 4u) {
            ctx->err = "pgs_prp_test: numbers above 4092 bits";
            return PGS_EINVAL;
        }
        if (bits <= 3) {  // 0..7: the reference's answers for 2, 3, 5, 7 are prime
            const uint32_t v0 = top ? v[0] : 0u;
            out[i] = (v0 == 2 || v0 == 3 || v0 == 5 || v0 == 7) ? 1 : 0;
            continue;
        }
        if (!(v[0] & 1u)) {
            out[i] = 0;
            continue;
        }
        max_bits = std::max(max_bits, bits);
        dev_rows.push_back(i);
    }
    if (dev_rows.empty()) return PGS_OK;
    const int L = pg::limbs_per_lane(max_bits);
    const uint32_t n = 8u * (uint32_t)L;
    std::vector<uint32_t> packed(dev_rows.size() * n, 0u);
    std::vector<pg::PrpItem> items(dev_rows.size());
    for (size_t j = 0; j < dev_rows.size(); j++) {
        const uint32_t *v = limbs + dev_rows[j] * n_limbs;
        std::memcpy(&packed[j * n], v, std::min(n, n_limbs) * 4u);
        items[j] = pg::PrpItem{(uint32_t)j, 0};
    }
    const cudaStream_t s = ctx->stream;
    DevBuf d_nums, d_items, d_res;
    DevBuf *bufs[] = {&d_nums, &d_items, &d_res};
    for (DevBuf *b : bufs) b->pool = &ctx->dpool;
    std::vector<uint8_t> res(dev_rows.size());
    cudaError_t e = upload(d_nums, packed, s);
    if (e == cudaSuccess) e = upload(d_items, items, s);
    if (e == cudaSuccess) e = d_res.ensure(dev_rows.size());
    if (e == cudaSuccess)
        e = pg::launch_prp(L, d_nums.as<uint32_t>(), d_items.as<pg::PrpItem>(), nullptr, dev_rows.size(),
                           d_res.as<uint8_t>(), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(res.data(), d_res.p, res.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamSynchronize(s);
    for (DevBuf *b : bufs) b->release();
    if (e != cudaSuccess) return fail(ctx, e, "pgs_prp_test");
    for (size_t j = 0; j < dev_rows.size(); j++) out[dev_rows[j]] = res[j];
    return PGS_OK;
}

}  // extern "C"

namespace {

// Device lists of rows (d_m .. d_dist, as pgs_unknowns) and the host copy of
// their m: the gap search.  The caller holds ctx->mu and checked the lists.
int prp_gaps_core(pgs_ctx *ctx, const pgs_gap_params *prm, uint64_t rows, const uint64_t *h_m,
                  const uint64_t *d_m, const uint64_t *d_start, const uint32_t *d_np, const uint32_t *d_nn,
                  const uint32_t *d_dist, pgs_gap_result *out, pgs_gap_stats *stats) {
    if (prm->p < 2 || !is_prime_u64(prm->p) || prm->d == 0 || prm->sieve_length == 0 ||
        prm->sieve_length >= (1u << 30)) {
        ctx->err = "pgs_prp_gaps: bad p, d or sieve_length";
        return PGS_EINVAL;
    }
    std::vector<uint32_t> k, kprimes;
    if (!build_k(prm->p, prm->d, k, kprimes) || (k.size() == 1 && k[0] <= 1)) {
        ctx->err = "pgs_prp_gaps: d does not divide p#";
        return PGS_EINVAL;
    }
    uint64_t max_m = 0;
    for (uint64_t r = 0; r < rows; r++) max_m = std::max(max_m, h_m[r]);
    const uint32_t bits = bits_of(k) + (64u - (uint32_t)__builtin_clzll(max_m)) + 1u;
    if (bits > 8u * pg::kMaxL * 32u - 4u) {
        ctx->err = "pgs_prp_gaps: m*K above 4092 bits";
        return PGS_EINVAL;
    }
    const int L = pg::limbs_per_lane(bits);
    const uint32_t n = 8u * (uint32_t)L;
    std::vector<uint32_t> skip(rows, 0u);
    if (prm->one_side_skip) {
        const double klog = k_log(k);
        for (uint64_t r = 0; r < rows; r++) skip[r] = skip_threshold(klog, h_m[r], prm->min_merit);
    }
    const cudaStream_t s = ctx->stream;
    DevBuf d_k, d_kp, d_skip, d_centers, d_state, d_items, d_res, d_out, d_ctr;
    DevBuf *bufs[] = {&d_k, &d_kp, &d_skip, &d_centers, &d_state, &d_items, &d_res, &d_out, &d_ctr};
    for (DevBuf *b : bufs) b->pool = &ctx->dpool;
    auto cleanup = [&] {
        cudaStreamSynchronize(s);
        for (DevBuf *b : bufs) b->release();
    };
    const uint64_t max_items = std::max<uint64_t>(rows, kRoundTarget + kMaxSpec);
    cudaError_t e = upload(d_k, k, s);
    if (e == cudaSuccess) e = upload(d_kp, kprimes, s);
    if (e == cudaSuccess) e = upload(d_skip, skip, s);
    if (e == cudaSuccess) e = d_centers.ensure(rows * n * 4ull);
    if (e == cudaSuccess) e = d_state.ensure(rows * sizeof(pg::GapRow));
    if (e == cudaSuccess) e = d_items.ensure(max_items * sizeof(pg::PrpItem));
    if (e == cudaSuccess) e = d_res.ensure(max_items);
    if (e == cudaSuccess) e = d_out.ensure(rows * sizeof(pgs_gap_result));
    if (e == cudaSuccess) e = d_ctr.ensure(32);
    if (e != cudaSuccess) {
        cleanup();
        return fail(ctx, e, "pgs_prp_gaps setup");
    }
    const pg::GapLists ls{d_start, d_np, d_nn, d_dist};
    unsigned long long *ctr = d_ctr.as<unsigned long long>();  // items, active, errors
    const unsigned rb = (unsigned)((rows + 255) / 256);
    pg::centers_kernel<<<rb, 256, 0, s>>>(d_k.as<uint32_t>(), (uint32_t)k.size(), d_m, rows, n,
                                          d_centers.as<uint32_t>());
    pg::gap_init_kernel<<<rb, 256, 0, s>>>(d_state.as<pg::GapRow>(), rows, ls, d_skip.as<uint32_t>(),
                                           d_centers.as<uint32_t>(), n, prm->sieve_length,
                                           d_out.as<pgs_gap_result>());
    e = cudaMemsetAsync(ctr, 0, 32, s);
    uint64_t active = rows, rounds = 0, launched = 0;
    uint64_t host_ctr[3] = {0, 0, 0};
    const uint32_t x_limit = prm->sieve_length + kPastScanSpan;
    while (e == cudaSuccess && active > 0) {
        const uint32_t spec =
            (uint32_t)std::min<uint64_t>(kMaxSpec, std::max<uint64_t>(1, kRoundTarget / active));
        e = cudaMemsetAsync(ctr, 0, 16, s);  // items, active
        if (e) break;
        pg::select_kernel<<<rb, 256, 0, s>>>(d_state.as<pg::GapRow>(), rows, ls, spec, d_kp.as<uint32_t>(),
                                             (uint32_t)kprimes.size(), x_limit, d_items.as<pg::PrpItem>(),
                                             max_items, ctr, ctr + 2);
        const uint64_t bound = std::min<uint64_t>(max_items, active * spec);
        e = pg::launch_prp(L, d_centers.as<uint32_t>(), d_items.as<pg::PrpItem>(), ctr, bound,
                           d_res.as<uint8_t>(), s);
        if (e) break;
        pg::resolve_kernel<<<rb, 256, 0, s>>>(d_state.as<pg::GapRow>(), rows, ls, d_items.as<pg::PrpItem>(),
                                              d_res.as<uint8_t>(), prm->sieve_length, d_out.as<pgs_gap_result>(),
                                              ctr + 1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(host_ctr, ctr, 24, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e) break;
        launched += host_ctr[0];
        active = host_ctr[1];
        if (++rounds > (1u << 22)) {
            cleanup();
            ctx->err = "pgs_prp_gaps: no progress";
            return PGS_ETIMEOUT;
        }
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out.p, rows * sizeof(pgs_gap_result), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) return fail(ctx, e, "pgs_prp_gaps");
    if (host_ctr[2]) {
        ctx->err = "pgs_prp_gaps: a side found no probable prime within 2^24 past the sieve length";
        return PGS_EABORT;
    }
    if (stats) {
        stats->rounds = rounds;
        stats->prp_tests = launched;
        stats->limbs = n;
    }
    return PGS_OK;
}

}  // namespace

extern "C" {

int pgs_prp_gaps(pgs_ctx *ctx, const pgs_gap_params *prm, const pgs_unknowns *lists, pgs_gap_result *out,
                 pgs_gap_stats *stats) {
    if (!ctx || !prm || !lists || (lists->rows && !out)) return PGS_EINVAL;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    const uint64_t rows = lists->rows;
    if (rows == 0) return PGS_OK;
    if (rows >= (1ull << 31) || !lists->m || !lists->start || !lists->n_prev || !lists->n_next ||
        (lists->total && !lists->dist)) {
        ctx->err = "pgs_prp_gaps: bad lists";
        return PGS_EINVAL;
    }
    for (uint64_t r = 0; r < rows; r++)
        if (lists->m[r] == 0 || lists->start[r] + lists->n_prev[r] + lists->n_next[r] > lists->total) {
            ctx->err = "pgs_prp_gaps: row outside the distance array";
            return PGS_EINVAL;
        }
    const cudaStream_t s = ctx->stream;
    PackedLists pk;
    pk.block.pool = &ctx->dpool;
    cudaError_t e = packed_alloc(pk, rows, lists->total);
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    if (e == cudaSuccess) e = up(pk.m, lists->m, rows * 8);
    if (e == cudaSuccess) e = up(pk.start, lists->start, rows * 8);
    if (e == cudaSuccess) e = up(pk.n_prev, lists->n_prev, rows * 4);
    if (e == cudaSuccess) e = up(pk.n_next, lists->n_next, rows * 4);
    if (e == cudaSuccess) e = up(pk.dist, lists->dist, lists->total * 4);
    int rc = e == cudaSuccess ? prp_gaps_core(ctx, prm, rows, lists->m, pk.m, pk.start, pk.n_prev, pk.n_next,
                                              pk.dist, out, stats)
                              : fail(ctx, e, "pgs_prp_gaps upload");
    cudaStreamSynchronize(s);
    pk.block.release();
    return rc;
}

int pgs_prp_gaps_prepared(pgs_ctx *ctx, pgs_prepared *prep, const pgs_gap_params *prm, pgs_gap_result *out,
                          pgs_gap_stats *stats) {
    if (!ctx || !prep || !prm || !out || prep->ctx != ctx || !prep->ran) return PGS_EINVAL;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    std::lock_guard<std::mutex> g(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    const HostJob &h = prep->hj;
    const uint64_t rows = h.valid_mi.size();
    if (rows == 0) return PGS_OK;
    std::vector<uint64_t> m(rows);
    for (uint64_t r = 0; r < rows; r++) m[r] = h.job.mstart + h.valid_mi[r];
    pgs_gap_params jp = *prm;  // the job's own p, d and sieve length
    jp.p = h.job.p;
    jp.d = h.job.d;
    jp.sieve_length = h.job.sieve_length;
    const cudaStream_t s = ctx->stream;
    PackedLists pk;
    int rc = job_lists_device(ctx, prep, s, pk);
    if (rc == PGS_OK)
        rc = prp_gaps_core(ctx, &jp, rows, m.data(), pk.m, pk.start, pk.n_prev, pk.n_next, pk.dist, out, stats);
    cudaStreamSynchronize(s);
    pk.block.release();
    return rc;
}

}  // extern "C"
