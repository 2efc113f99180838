// Large-prime phase: for every prime p > 4*SL+2, every m in
// [mstart, mstart+minc) and offset X in [-SL, SL] with p | m*K + X and
// m*K + X odd (the parity-reduced walk of WalkParams, pg_arith.cuh).
//
// Replaces method2_large_primes (combined_sieve.cpp:1763-2011) and the
// enumeration modulo_search_euclid_all_large (modulo_search.cpp:339-376).
// With y(mi) = (r*(mstart+mi) + SL) mod p, r = K mod p, a hit is y <= 2*SL and
// marks offset X = SL - y of m = mstart + mi.
//
// The reference runs one Euclid modulo search per hit.  Here one continued
// fraction per prime (pg::first_entry) yields both the first hit and the
// last level (kp, up, kn, dn) of a Rauzy induction of y -> y + r (mod p); after
// the first hit, the walk is a rotation by `up` on a circle of C = up + dn
// points, every step costing kp or kn in mi, and every point below 2*SL+1 is a
// hit.  Step n has the closed form Y = y0 + n*up, residue Y mod C, so a prime's
// steps split into independent items with no further search.
//
// Scheduling: a persistent grid whose CTAs claim groups of 256 primes from an
// atomic counter (the prime list is roughly ascending, so the heavy small
// primes go first).  Phase 1 (one thread per prime) runs the continued
// fraction; primes with few steps finish right there, primes with very many
// steps (the smallest ones) go to a device list for heavy_kernel, one CTA per
// prime, and the rest publish their rotation in shared memory for phase 2,
// which spreads their steps over the CTA in items (2^item_shift steps; the
// three step thresholds are the job's tuning, JobDev).  Hits go
// through a valid-m bitmask and a live-offset bitmask held in shared memory;
// only the survivors (a few percent) take their bitset row and column as
// ranks in those masks (rank counts beside them, no table reads) and set one
// bit of the L2-resident composite bitset with a global atomicOr.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "pg_arith.cuh"
#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kLargeThreads = 256;

// A walk hit (j, Y) is m = mstart + mi_base + stride*j, x = X + SL = xc - 2Y.
// The masks are indexed by j and Y and stored as {bits, set bits before the
// word} pairs, so one 64-bit read per mask gives both a hit's filter bits and,
// for a survivor, its bitset row (rank of j among the valid m) and column
// (from ry, the live Y below Y: ry - H for X < 0, Hp + H - 1 - ry above).
struct Marker {
    const JobDev &job;
    const uint2 *mmask;  // valid m over j (shared or global)
    const uint2 *ymask;  // live offsets over Y
    // Called at every walk step (hit or not) with j < jmax; the mask pairs
    // are read unconditionally (Y = 0 stands in off a hit) and only a
    // surviving hit branches to the atomic.
    __device__ __forceinline__ void operator()(uint64_t j64, uint32_t y, bool hit) const {
        const uint32_t j = (uint32_t)j64, yi = hit ? y : 0u;
        const uint2 yv = ymask[yi >> 5], mv = mmask[j >> 5];
        const uint32_t yb = (yv.x >> (yi & 31)) & 1u;
        const uint32_t mb = (mv.x >> (j & 31)) & 1u;
        if (hit & (yb & mb)) {
            const uint32_t row = mv.y + __popc(mv.x & ((1u << (j & 31)) - 1u));
            const uint32_t ry = yv.y + __popc(yv.x & ((1u << (yi & 31)) - 1u));
            const uint32_t col = yi >= job.y_lo ? ry - job.half_cols : job.side_pad + job.half_cols - 1 - ry;
            if (job.mark_mode == kMarkComp) {
                atomicOr(&job.comp[(uint64_t)row * job.pitch + (col >> 5)], 1u << (col & 31));
            } else if (job.mark_mode == kMarkCount) {
                atomicAdd(&job.row_count[row], 1ull);
            } else {
                const unsigned long long k = atomicAdd(&job.row_count[row], 1ull);
                job.bucket[job.row_off[row] + k] = col;
            }
        }
    }
};

}  // namespace

struct HeavyPrime {
    uint32_t mi0, y0, up, dn;
    uint64_t kp, kn, steps;
    uint32_t job, pad;  // job index in a multi-job launch (0 for one job)
};
static_assert(sizeof(HeavyPrime) == kHeavyPrimeBytes, "heavy list stride");

// A walk of more than direct_steps and at most heavy_steps steps, handed from
// the warp-alone continued-fraction kernel to walk_kernel: first hit
// (mi0, y0) and the rotation, step costs clamped to the walk's end (gap32).
struct WalkEntry {
    uint32_t mi0, y0, up, dn, kp, kn, steps, pad;
};
static_assert(sizeof(WalkEntry) == kWalkEntryBytes, "walk list stride");

namespace {

template <typename T>
struct Slots {
    uint32_t mi0[kLargeThreads];
    uint32_t y0[kLargeThreads];
    uint32_t up[kLargeThreads];
    uint32_t dn[kLargeThreads];
    T kp[kLargeThreads];
    T kn[kLargeThreads];
    uint32_t start[kLargeThreads + 1];
    uint32_t warp_total[kLargeThreads / 32];
};

// Words of the two masks: valid m over walk indices, live offsets over
// walk residues.
__host__ __device__ inline uint32_t mask_words_m(const JobDev &job) { return (uint32_t)((job.walk.jmax + 31) / 32); }
__host__ __device__ inline uint32_t mask_words_y(const JobDev &job) { return (job.walk.w + 31) / 32; }

// Copies the masks ({bits, rank} pairs) to shared memory when they fit
// (kShared, a template parameter so that every mask read of a walk step
// compiles to a shared-memory load rather than a generic one); returns where
// the kernel reads them.
template <bool kShared>
__device__ __forceinline__ void load_masks(const JobDev &job, const uint2 *g_mmask, const uint2 *g_ymask,
                                           uint2 *s_masks, const uint2 *&mmask, const uint2 *&ymask) {
    if constexpr (kShared) {
        const uint32_t mwords = mask_words_m(job), ywords = mask_words_y(job);
        for (uint32_t i = threadIdx.x; i < mwords; i += blockDim.x) s_masks[i] = g_mmask[i];
        for (uint32_t i = threadIdx.x; i < ywords; i += blockDim.x) s_masks[mwords + i] = g_ymask[i];
        mmask = s_masks;
        ymask = s_masks + mwords;
    } else {
        mmask = g_mmask;
        ymask = g_ymask;
    }
    __syncthreads();
}

// Where a kernel's walk inputs come from.
constexpr int kInWalk = 0;      // a = the job's walk step, b = its start residue (kmod_window)
constexpr int kInKprime = 1;    // a = K' mod p, b = R^2 mod p: the walk of K = K' * kmul starts here
constexpr int kInLimbsLsb = 2;  // K mod p computed here from K's limbs, least significant first
constexpr int kInLimbsMsb = 3;  // the same, most significant limb first

// Walk step and start residue of prime p, the i-th of the window's inputs
// a_in, b_in (kInWalk, kInKprime), or of K's limbs (kInLimbs*: one thread
// per prime does K mod p here, so the large-prime phase's continued
// fractions, mostly integer-ALU work, share the SM with the K mod p chains,
// mostly wide multiplies, instead of following them in another launch).
template <typename T, int kIn>
__device__ __forceinline__ void walk_inputs(const JobDev &job, const uint32_t *limbs, int nlimbs, T p,
                                            const T *a_in, const T *b_in, uint64_t i, T &step, T &t0) {
    if constexpr (kIn == kInWalk) {
        step = a_in[i];
        t0 = b_in[i];
    } else if constexpr (kIn == kInKprime) {
        if constexpr (sizeof(T) == 4)
            walk_start(job.walk, p, a_in[i], b_in[i], step, t0, job.kmul);
        else
            walk_start(job.walk, p, a_in[i], neg_inv64(p), b_in[i], step, t0, job.kmul);
    } else if constexpr (sizeof(T) == 4) {
        uint32_t pp[1] = {p}, r[1], pinv[1], r2[1];
        if constexpr (kIn == kInLimbsLsb)
            kmod32_lsb_multi<1>(limbs, nlimbs, pp, r, pinv, r2);
        else
            kmod32_multi<1>(limbs, nlimbs, pp, r, pinv, r2);
        walk_start(job.walk, p, r[0], r2[0], step, t0, 1, pinv[0]);
    } else {
        uint64_t pinv, r2;
        const uint64_t r = kIn == kInLimbsLsb ? kmod64_lsb(limbs, nlimbs, p, &pinv, &r2)
                                              : kmod64(limbs, nlimbs, p, &pinv, &r2);
        walk_start(job.walk, p, r, pinv, r2, step, t0);
    }
}

// One group of up to kLargeThreads primes of one job; the whole CTA calls it.
// has: this thread holds a prime p with its walk step and start residue t0.
// Phase 1 runs each prime's continued fraction; few steps are walked at
// once, very many go to the heavy list (tagged with job_tag), the rest are
// spread over the CTA as items of 2^job.item_shift steps (phase 2).
template <typename T>
__device__ __forceinline__ void large_group(const JobDev &job, const Marker &mark, Slots<T> &sl, bool has,
                                            T p, T step, T t0, HeavyPrime *heavy,
                                            unsigned long long *heavy_count, uint32_t heavy_cap,
                                            uint32_t job_tag) {
    const T w = (T)job.walk.w;
    const uint64_t minc = job.walk.jmax;  // the walk runs over j, not mi
    uint32_t items = 0;
    if (has) {
        const Entry<T> e = first_entry<T>(p, step, w, t0, minc);
        if (e.t < minc && e.y < w) {
            const uint64_t bound = rotation_steps_bound<T>(e.t, minc, e.g, p);
            bool local = true;
            if (bound <= job.direct_steps) {
                // few steps: walk the rotation here
                return_walk32((uint32_t)e.t, (uint32_t)e.y, gap32(e.g, (uint32_t)minc), (uint32_t)w,
                                (uint32_t)minc, (uint32_t)bound, mark);
                local = false;
            } else if (bound > job.heavy_steps) {
                // very many steps: one CTA of the heavy kernel takes this prime
                const unsigned long long h = atomicAdd(heavy_count, 1ull);
                if (h < heavy_cap) {
                    heavy[h] = HeavyPrime{(uint32_t)e.t, (uint32_t)e.y, (uint32_t)e.g.up,
                                          (uint32_t)e.g.dn, (uint64_t)e.g.kp,
                                          (uint64_t)e.g.kn, bound, job_tag, 0u};
                    local = false;
                }
            }
            if (local) {
                sl.mi0[threadIdx.x] = (uint32_t)e.t;
                sl.y0[threadIdx.x] = (uint32_t)e.y;
                sl.up[threadIdx.x] = (uint32_t)e.g.up;
                sl.dn[threadIdx.x] = (uint32_t)e.g.dn;
                sl.kp[threadIdx.x] = e.g.kp;
                sl.kn[threadIdx.x] = e.g.kn;
                items = (uint32_t)((bound + (1u << job.item_shift) - 1) >> job.item_shift);
            }
        }
    }
    // exclusive scan of item counts (skipped when the group has none):
    // shuffle scan within each warp, then the warps' totals
    if (!__syncthreads_or(items != 0)) return;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = items;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31) sl.warp_total[warp] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int k = 0; k < kLargeThreads / 32; k++) {
        const uint32_t t = sl.warp_total[k];
        before += k < (int)warp ? t : 0u;
        total += t;
    }
    sl.start[threadIdx.x + 1] = before + incl;
    if (threadIdx.x == 0) sl.start[0] = 0;
    __syncthreads();
    for (uint32_t it = threadIdx.x; it < total; it += kLargeThreads) {
        uint32_t lo = 0, hi = kLargeThreads;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (sl.start[mid] <= it) lo = mid;
            else hi = mid;
        }
        const uint32_t s = lo;
        const uint32_t shift = job.item_shift;
        const uint64_t n0 = (uint64_t)(it - sl.start[s]) << shift;
        const ThreeGap<uint32_t> g =
            gap32(ThreeGap<T>{sl.kp[s], (T)sl.up[s], sl.kn[s], (T)sl.dn[s]}, (uint32_t)minc);
        uint32_t y, mi;
        rotation_at32(sl.mi0[s], sl.y0[s], g, (uint32_t)n0, (uint32_t)minc, y, mi);
        return_walk32(mi, y, g, (uint32_t)w, (uint32_t)minc, 1u << shift, mark);
    }
    __syncthreads();
}

template <typename T, int kIn, bool kShared>
__global__ void __launch_bounds__(kLargeThreads, sizeof(T) == 4 ? 8 : 1)
    large_kernel(const __grid_constant__ KLimbs<kIn >= kInLimbsLsb ? kParamLimbs : 1> kl, int nlimbs,
                 JobDev job, uint64_t base, const uint32_t *__restrict__ off,
                 const unsigned long long *range, uint64_t max_count, const T *__restrict__ a_in,
                 const void *__restrict__ b_in, const unsigned long long *rrange,
                 const uint2 *__restrict__ g_mmask,
                 const uint2 *__restrict__ g_ymask,
                 unsigned long long *group_ctr, HeavyPrime *heavy, unsigned long long *heavy_count,
                 uint32_t heavy_cap) {
    extern __shared__ uint2 s_masks[];
    __shared__ Slots<T> sl;
    __shared__ unsigned long long s_group;
    const uint2 *mmask, *ymask;
    load_masks<kShared>(job, g_mmask, g_ymask, s_masks, mmask, ymask);
    const Marker mark{job, mmask, ymask};
    const uint64_t n = min((uint64_t)(range[1] - range[0]), max_count);
    off += range[0];
    const T *b = (const T *)b_in;  // R^2 mod p, or the start residue
    if constexpr (kIn < kInLimbsLsb) {
        a_in += range[0] - rrange[0];
        b += range[0] - rrange[0];
    }

    for (;;) {
        if (threadIdx.x == 0) s_group = atomicAdd(group_ctr, 1ull);
        __syncthreads();
        const uint64_t group = s_group;
        if (group * kLargeThreads >= n) break;
        const uint64_t i = group * kLargeThreads + threadIdx.x;
        const bool has = i < n;
        const T p = has ? (T)(base + off[i]) : (T)0;
        T step = 0, t0 = 0;
        if (has) walk_inputs<T, kIn>(job, kl.limb, nlimbs, p, a_in, b, i, step, t0);
        large_group<T>(job, mark, sl, has, p, step, t0, heavy, heavy_count, heavy_cap, 0u);
    }
}

// Many jobs in one launch: CTAs claim tiles of kLargeThreads primes from a
// device counter over the items (a job's primes in one prime-table window,
// items in job order, tiles numbered consecutively), load the job's masks
// into shared memory when the tile's job differs from their last one, and
// run the group as the single-job kernel does, with the job's walk started
// from K' mod p.  Every item has the same prime width (T).
template <typename T, bool kAllShared>
__global__ void __launch_bounds__(kLargeThreads, sizeof(T) == 4 ? 8 : 1)
    large_multi_kernel(const LargeJob *__restrict__ jobs, const LargeItem *__restrict__ items, uint32_t n_items,
                       uint32_t n_tiles, unsigned long long *tile_ctr, HeavyPrime *heavy,
                       unsigned long long *heavy_count, uint32_t heavy_cap) {
    extern __shared__ uint2 s_masks[];
    __shared__ Slots<T> sl;
    __shared__ JobDev s_job;
    __shared__ uint32_t s_tile, s_item;
    __shared__ const uint2 *s_mm, *s_ym;
    uint32_t loaded = ~0u;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t t = (uint32_t)atomicAdd(tile_ctr, 1ull);
            s_tile = t;
            if (t < n_tiles) {
                uint32_t lo = 0, hi = n_items;  // last item with tile0 <= t
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (items[mid].tile0 <= t) lo = mid;
                    else hi = mid;
                }
                s_item = lo;
            }
        }
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= n_tiles) break;
        const LargeItem &it = items[s_item];
        if (it.job != loaded) {
            // another job: its descriptor and masks (all threads passed the
            // barrier above, so nobody still reads the old ones)
            const LargeJob &lj = jobs[it.job];
            if (threadIdx.x == 0) s_job = lj.job;
            const uint32_t mwords = (uint32_t)((lj.job.walk.jmax + 31) / 32), ywords = (lj.job.walk.w + 31) / 32;
            if (kAllShared || lj.masks_in_shared) {
                for (uint32_t i = threadIdx.x; i < mwords; i += blockDim.x) s_masks[i] = lj.mmask[i];
                for (uint32_t i = threadIdx.x; i < ywords; i += blockDim.x) s_masks[mwords + i] = lj.ymask[i];
                if (threadIdx.x == 0) s_mm = s_masks, s_ym = s_masks + mwords;
            } else if (threadIdx.x == 0) {
                s_mm = lj.mmask, s_ym = lj.ymask;
            }
            loaded = it.job;
            __syncthreads();
        }
        const uint32_t i = (t - it.tile0) * kLargeThreads + threadIdx.x;
        const bool has = i < it.count;
        const T *a = (const T *)it.a, *b = (const T *)it.b;
        const T p = has ? (T)(it.base + it.off[i]) : (T)0;
        T step = 0, t0 = 0;
        if (has) walk_inputs<T, kInKprime>(s_job, nullptr, 0, p, a, b, i, step, t0);
        if constexpr (kAllShared) {
            // every job's masks in shared memory: shared loads (see load_masks)
            const Marker mark{s_job, s_masks, s_masks + (uint32_t)((s_job.walk.jmax + 31) / 32)};
            large_group<T>(s_job, mark, sl, has, p, step, t0, heavy, heavy_count, heavy_cap, it.job);
        } else {
            const Marker mark{s_job, s_mm, s_ym};
            large_group<T>(s_job, mark, sl, has, p, step, t0, heavy, heavy_count, heavy_cap, it.job);
        }
    }
}

// The warp-alone form of one job (tuning knob large_form, bit 0): no CTA
// barrier after the masks.  Each warp claims 32 primes at a time, runs their
// continued fractions, walks the short rotations (at most direct_steps
// steps) in place and hands the others to two lists -- up to heavy_steps
// steps to walk_kernel (one warp per walk), more to heavy_kernel (one CTA per
// prime).  A full list falls back to the next one, and finally to walking the
// rotation in this thread.  Faster than the pooled form when walks are short
// (small jobs: P = 503, SL = 5e3, 1e4 m, primes to 1e8: large stage 0.43 ->
// 0.35 ms), slower when many walks of 25-100 steps leave each lane of
// walk_kernel only a few steps after its closed-form start (P = 1511,
// SL = 2e4, 1e5 m, primes to 2e9: 5.85 -> 8.64 ms); the tuner picks per class.
template <typename T, int kIn, bool kShared>
__global__ void __launch_bounds__(kLargeThreads)
    large_cf_kernel(const __grid_constant__ KLimbs<kIn >= kInLimbsLsb ? kParamLimbs : 1> kl, int nlimbs,
                    JobDev job, uint64_t base, const uint32_t *__restrict__ off,
                    const unsigned long long *range, uint64_t max_count, const T *__restrict__ a_in,
                    const void *__restrict__ b_in, const unsigned long long *rrange,
                    const uint2 *__restrict__ g_mmask, const uint2 *__restrict__ g_ymask,
                    unsigned long long *ctr, HeavyPrime *heavy, uint32_t heavy_cap, WalkEntry *walks,
                    uint32_t walk_cap) {
    extern __shared__ uint2 s_masks[];
    const uint2 *mmask, *ymask;
    load_masks<kShared>(job, g_mmask, g_ymask, s_masks, mmask, ymask);
    const Marker mark{job, mmask, ymask};
    const uint64_t n = min((uint64_t)(range[1] - range[0]), max_count);
    off += range[0];
    const T *b = (const T *)b_in;
    if constexpr (kIn < kInLimbsLsb) {
        a_in += range[0] - rrange[0];
        b += range[0] - rrange[0];
    }
    const T w = (T)job.walk.w;
    const uint64_t minc = job.walk.jmax;
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long g = 0;
        if (lane == 0) g = atomicAdd(ctr, 1ull);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g * 32 >= n) break;
        const uint64_t i = g * 32 + lane;
        if (i >= n) continue;
        const T p = (T)(base + off[i]);
        T step, t0;
        walk_inputs<T, kIn>(job, kl.limb, nlimbs, p, a_in, b, i, step, t0);
        const Entry<T> e = first_entry<T>(p, step, w, t0, minc);
        if (e.t >= minc || e.y >= w) continue;
        const uint64_t bound = rotation_steps_bound<T>(e.t, minc, e.g, p);
        const ThreeGap<uint32_t> g32 = gap32(e.g, (uint32_t)minc);
        if (bound > job.direct_steps) {
            if (bound <= job.heavy_steps) {
                const unsigned long long k = atomicAdd(ctr + 2, 1ull);
                if (k < walk_cap) {
                    walks[k] = WalkEntry{(uint32_t)e.t, (uint32_t)e.y, g32.up, g32.dn, g32.kp, g32.kn,
                                         (uint32_t)bound, 0u};
                    continue;
                }
            }
            const unsigned long long h = atomicAdd(ctr + 1, 1ull);
            if (h < heavy_cap) {
                heavy[h] = HeavyPrime{(uint32_t)e.t, (uint32_t)e.y, (uint32_t)e.g.up, (uint32_t)e.g.dn,
                                      (uint64_t)e.g.kp, (uint64_t)e.g.kn, bound, 0u, 0u};
                continue;
            }
        }
        return_walk32((uint32_t)e.t, (uint32_t)e.y, g32, (uint32_t)w, (uint32_t)minc, (uint32_t)bound, mark);
    }
}

// The walk list of the warp-alone form: each warp claims one walk and splits
// its steps evenly over its lanes (each lane starts from the closed form).
template <bool kShared>
__global__ void __launch_bounds__(kLargeThreads)
    walk_kernel(JobDev job, const WalkEntry *__restrict__ walks, const unsigned long long *ctr, uint32_t walk_cap,
                const uint2 *__restrict__ g_mmask, const uint2 *__restrict__ g_ymask, unsigned long long *claim) {
    extern __shared__ uint2 s_masks[];
    const uint2 *mmask, *ymask;
    load_masks<kShared>(job, g_mmask, g_ymask, s_masks, mmask, ymask);
    const Marker mark{job, mmask, ymask};
    const uint64_t nw = min((uint64_t)ctr[2], (uint64_t)walk_cap);
    const uint32_t jmax = (uint32_t)job.walk.jmax, w = job.walk.w, lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(claim, 1ull);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= nw) break;
        const WalkEntry we = walks[k];
        const ThreeGap<uint32_t> g{we.kp, we.up, we.kn, we.dn};
        const uint32_t per = (we.steps + 31) / 32, n0 = lane * per;
        if (n0 >= we.steps) continue;
        uint32_t y, mi;
        rotation_at32(we.mi0, we.y0, g, n0, jmax, y, mi);
        return_walk32(mi, y, g, w, jmax, per, mark);
    }
}

// One CTA per heavy prime: its rotation steps split over the CTA's threads.
template <bool kShared>
__global__ void __launch_bounds__(kLargeThreads)
    heavy_kernel(JobDev job, const HeavyPrime *__restrict__ heavy,
                 const unsigned long long *heavy_count, uint32_t heavy_cap,
                 const uint2 *__restrict__ g_mmask, const uint2 *__restrict__ g_ymask) {
    extern __shared__ uint2 s_masks[];
    const uint2 *mmask, *ymask;
    load_masks<kShared>(job, g_mmask, g_ymask, s_masks, mmask, ymask);
    const Marker mark{job, mmask, ymask};
    const uint64_t nh = min((uint64_t)*heavy_count, (uint64_t)heavy_cap);
    const uint32_t w = job.walk.w;
    for (uint64_t h = blockIdx.x; h < nh; h += gridDim.x) {
        const HeavyPrime hp = heavy[h];
        const uint32_t jmax = (uint32_t)job.walk.jmax, shift = job.item_shift;
        const ThreeGap<uint32_t> g = gap32(ThreeGap<uint64_t>{hp.kp, hp.up, hp.kn, hp.dn}, jmax);
        const uint64_t items = (hp.steps + (1u << shift) - 1) >> shift;
        for (uint64_t it = threadIdx.x; it < items; it += blockDim.x) {
            uint32_t y, mi;
            rotation_at32(hp.mi0, hp.y0, g, (uint32_t)(it << shift), jmax, y, mi);
            return_walk32(mi, y, g, w, jmax, 1u << shift, mark);
        }
    }
}

// Heavy primes of many jobs: each entry carries its job; the masks are read
// from global memory (L2), since consecutive entries of one CTA belong to
// different jobs.
__global__ void __launch_bounds__(kLargeThreads)
    heavy_multi_kernel(const LargeJob *__restrict__ jobs, const HeavyPrime *__restrict__ heavy,
                       const unsigned long long *heavy_count, uint32_t heavy_cap) {
    __shared__ JobDev s_job;
    __shared__ uint32_t s_loaded;
    if (threadIdx.x == 0) s_loaded = ~0u;
    const uint64_t nh = min((uint64_t)*heavy_count, (uint64_t)heavy_cap);
    for (uint64_t h = blockIdx.x; h < nh; h += gridDim.x) {
        const HeavyPrime hp = heavy[h];
        __syncthreads();
        if (threadIdx.x == 0 && s_loaded != hp.job) {
            s_job = jobs[hp.job].job;
            s_loaded = hp.job;
        }
        __syncthreads();
        const LargeJob &lj = jobs[hp.job];
        const Marker mark{s_job, lj.mmask, lj.ymask};
        const uint32_t jmax = (uint32_t)s_job.walk.jmax, w = s_job.walk.w, shift = s_job.item_shift;
        const ThreeGap<uint32_t> g = gap32(ThreeGap<uint64_t>{hp.kp, hp.up, hp.kn, hp.dn}, jmax);
        const uint64_t items = (hp.steps + (1u << shift) - 1) >> shift;
        for (uint64_t it = threadIdx.x; it < items; it += blockDim.x) {
            uint32_t y, mi;
            rotation_at32(hp.mi0, hp.y0, g, (uint32_t)(it << shift), jmax, y, mi);
            return_walk32(mi, y, g, w, jmax, 1u << shift, mark);
        }
    }
}

}  // namespace

uint32_t heavy_capacity() { return 1u << 20; }
uint32_t walk_capacity() { return 1u << 24; }

namespace {

// One CTA per row of the per-m path: the row's survivor columns, in any
// order and with repeats, set bits of its comp row in shared memory, which
// then replaces the (zeroed) comp row.
constexpr int kApplyThreads = 256;
__global__ void __launch_bounds__(kApplyThreads)
    bucket_apply_kernel(JobDev job, const unsigned long long *__restrict__ total) {
    extern __shared__ uint32_t s_row[];
    const uint32_t row = blockIdx.x;
    for (uint32_t w = threadIdx.x; w < job.pitch; w += blockDim.x) s_row[w] = 0;
    __syncthreads();
    const unsigned long long b0 = job.row_off[row];
    const unsigned long long b1 = row + 1 < job.rows ? job.row_off[row + 1] : *total;
    for (unsigned long long k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
        const uint32_t col = job.bucket[k];
        atomicOr(&s_row[col >> 5], 1u << (col & 31));
    }
    __syncthreads();
    uint32_t *dst = job.comp + (uint64_t)row * job.pitch;
    for (uint32_t w = threadIdx.x; w < job.pitch; w += blockDim.x) dst[w] = s_row[w];
}

}  // namespace

cudaError_t bucket_apply(const JobDev &job, const unsigned long long *total, cudaStream_t stream) {
    if (job.rows == 0) return cudaSuccess;
    const size_t smem = (size_t)job.pitch * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(bucket_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e) return e;
    bucket_apply_kernel<<<job.rows, kApplyThreads, smem, stream>>>(job, total);
    return cudaGetLastError();
}

cudaError_t large_window(const JobDev &job, uint64_t base, const uint32_t *d_off,
                         const unsigned long long *d_range, uint64_t max_count, const void *d_a,
                         const void *d_b, const unsigned long long *d_rrange, bool wide,
                         bool start_in_kernel, const uint2 *d_mmask, const uint2 *d_ymask,
                         LargeScratch scratch, cudaStream_t stream, const uint32_t *h_klimbs, int nlimbs,
                         bool lsb) {
    if (max_count == 0) return cudaSuccess;
    const size_t mask_bytes = 8ull * (mask_words_m(job) + mask_words_y(job));
    const int in_shared = mask_bytes <= 96 * 1024;
    const size_t smem = in_shared ? mask_bytes : 0;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e;
    if ((e = cudaMemsetAsync(scratch.counters, 0, kLargeCounters * sizeof(unsigned long long), stream))) return e;
    unsigned long long *group_ctr = scratch.counters, *heavy_count = scratch.counters + 1;
    // K's limbs in the launch's parameters when the kernel reduces K itself
    const bool fused = h_klimbs != nullptr && nlimbs >= 1 && nlimbs <= kParamLimbs;
    KLimbs<kParamLimbs> klp;
    const KLimbs<1> kl1{};
    if (fused) memcpy(klp.limb, h_klimbs, (size_t)nlimbs * sizeof(uint32_t));
    if (!fused && d_rrange == nullptr) return cudaErrorInvalidValue;
    auto prep = [&](auto kernel) -> cudaError_t {
        // static + dynamic shared memory above 48 KiB needs the opt-in, and
        // the kernels' static part is several KiB: always state the size
        cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err) return err;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kLargeThreads, smem);
        return cudaSuccess;
    };
    auto launch = [&](auto kernel, const auto &kl, const auto *a) -> cudaError_t {
        cudaError_t err = prep(kernel);
        if (err) return err;
        if (per_sm < 1) per_sm = 1;
        const uint64_t groups = (max_count + kLargeThreads - 1) / kLargeThreads;
        uint64_t blocks = (uint64_t)sms * per_sm;
        if (blocks > groups) blocks = groups;
        kernel<<<(unsigned)blocks, kLargeThreads, smem, stream>>>(
            kl, nlimbs, job, base, d_off, d_range, max_count, a, d_b, d_rrange, d_mmask, d_ymask,
            group_ctr, scratch.heavy, heavy_count, scratch.heavy_cap);
        return cudaSuccess;
    };
    // the warp-alone form: as many warps as fit, each claiming 32 primes
    auto launch_cf = [&](auto kernel, const auto &kl, const auto *a) -> cudaError_t {
        cudaError_t err = prep(kernel);
        if (err) return err;
        if (per_sm < 1) per_sm = 1;
        const uint64_t ctas = ((max_count + 31) / 32 + kLargeThreads / 32 - 1) / (kLargeThreads / 32);
        const uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, ctas);
        kernel<<<(unsigned)blocks, kLargeThreads, smem, stream>>>(
            kl, nlimbs, job, base, d_off, d_range, max_count, a, d_b, d_rrange, d_mmask, d_ymask,
            scratch.counters, scratch.heavy, scratch.heavy_cap, scratch.walks, scratch.walk_cap);
        return cudaSuccess;
    };
    const bool alone = (job.large_form & 1u) && scratch.walks != nullptr;
    // kernel form x prime width x where the walk inputs come from x where the masks live
    auto pick = [&](auto t, auto sh) -> cudaError_t {
        using T = decltype(t);
        constexpr bool S = decltype(sh)::value;
        const T *a = (const T *)d_a;
        if (fused) {
            if (alone)
                return lsb ? launch_cf(large_cf_kernel<T, kInLimbsLsb, S>, klp, a)
                           : launch_cf(large_cf_kernel<T, kInLimbsMsb, S>, klp, a);
            return lsb ? launch(large_kernel<T, kInLimbsLsb, S>, klp, a)
                       : launch(large_kernel<T, kInLimbsMsb, S>, klp, a);
        }
        if (alone)
            return start_in_kernel ? launch_cf(large_cf_kernel<T, kInKprime, S>, kl1, a)
                                   : launch_cf(large_cf_kernel<T, kInWalk, S>, kl1, a);
        return start_in_kernel ? launch(large_kernel<T, kInKprime, S>, kl1, a)
                               : launch(large_kernel<T, kInWalk, S>, kl1, a);
    };
    auto walks_heavy = [&](auto sh) -> cudaError_t {
        constexpr bool S = decltype(sh)::value;
        cudaError_t err;
        if (alone) {
            if ((err = prep(walk_kernel<S>))) return err;
            if (per_sm < 1) per_sm = 1;
            walk_kernel<S><<<(unsigned)(sms * per_sm), kLargeThreads, smem, stream>>>(
                job, scratch.walks, scratch.counters, scratch.walk_cap, d_mmask, d_ymask, scratch.counters + 3);
            if ((err = cudaGetLastError())) return err;
        }
        if ((err = prep(heavy_kernel<S>))) return err;
        if (per_sm < 1) per_sm = 1;
        heavy_kernel<S><<<(unsigned)(sms * per_sm), kLargeThreads, smem, stream>>>(
            job, scratch.heavy, heavy_count, scratch.heavy_cap, d_mmask, d_ymask);
        return cudaGetLastError();
    };
    using Shared = std::true_type;
    using Global = std::false_type;
    if (in_shared)
        e = wide ? pick(uint64_t{}, Shared{}) : pick(uint32_t{}, Shared{});
    else
        e = wide ? pick(uint64_t{}, Global{}) : pick(uint32_t{}, Global{});
    if (e) return e;
    if ((e = cudaGetLastError())) return e;
    return in_shared ? walks_heavy(Shared{}) : walks_heavy(Global{});
}

cudaError_t large_multi(const LargeJob *d_jobs, const LargeItem *d_items, uint32_t n_items, uint32_t n_tiles,
                        size_t smem, bool wide, LargeScratch scratch, cudaStream_t stream, bool all_shared) {
    if (n_tiles == 0) return cudaSuccess;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e;
    if ((e = cudaMemsetAsync(scratch.counters, 0, 2 * sizeof(unsigned long long), stream))) return e;
    unsigned long long *tile_ctr = scratch.counters, *heavy_count = scratch.counters + 1;
    auto launch = [&](auto kernel) -> cudaError_t {
        cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err) return err;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kLargeThreads, smem);
        if (per_sm < 1) per_sm = 1;
        const uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, n_tiles);
        kernel<<<(unsigned)blocks, kLargeThreads, smem, stream>>>(d_jobs, d_items, n_items, n_tiles, tile_ctr,
                                                                  scratch.heavy, heavy_count, scratch.heavy_cap);
        return cudaGetLastError();
    };
    if (all_shared)
        e = wide ? launch(large_multi_kernel<uint64_t, true>) : launch(large_multi_kernel<uint32_t, true>);
    else
        e = wide ? launch(large_multi_kernel<uint64_t, false>) : launch(large_multi_kernel<uint32_t, false>);
    if (e) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, heavy_multi_kernel, kLargeThreads, 0))) return e;
    if (per_sm < 1) per_sm = 1;
    heavy_multi_kernel<<<(unsigned)(sms * per_sm), kLargeThreads, 0, stream>>>(d_jobs, scratch.heavy, heavy_count,
                                                                               scratch.heavy_cap);
    return cudaGetLastError();
}

}  // namespace pg
