// exact_runs.cuh - the sequential double sum of nonnegative terms (the problem of exact_sum.cuh)
// by predicted binade runs.
//
// An approximate prefix sum, taken in any order, places every partial sum of the sequence in
// its binade up to a relative margin (about 1.5e-8: the sequential sum of k terms is within
// k 2^-53 of the exact one, the approximate prefix far closer). Terms whose partial sums before
// and after lie safely inside one binade form runs; the increment pairs of a run's terms (exact_sum.cuh:
// integer additions in the binade's ulps, ties keyed by parity) compose into one pair in
// parallel. A term at which the binade may change is a single, added by the hardware. One thread
// then walks the segments in order with the exact running sum: a run is applied in one step when
// the running sum is in the run's binade and stays below the binade's top, and otherwise (a
// wrong prediction) summed term by term by exact::sequential_sum_from. The predictions only
// choose the path; every step is the sequential sum's own rounding.
//
// A tile of kTile terms is one block's work: its segments go to a region of kTileSegs records;
// a tile with more segments than that is marked and summed term by term by the walk.
#pragma once

#include <cstdint>

#include "exact_sum.cuh"

namespace svxg {
namespace exact {

constexpr int64_t kTile = int64_t(kThreads) * kItems;  // terms per tile (one block)
constexpr int32_t kTileSegs = 1024;                     // segment records per tile
constexpr int32_t kSkipCode = 100000;    // zeros before the first nonzero term: no change
constexpr int32_t kSingleCode = 100001;  // one term, added by the hardware
constexpr int32_t kRangeCode = 100002;   // a tile summed term by term (walk only)
constexpr int64_t kTop = int64_t(1) << 53;

struct Seg {
  Pair pair;      // a run: the composed increments in ulps of 2^code
  double t;       // a single: the term
  int64_t first;  // the segment's first term
  int32_t count;  // its terms
  int32_t code;   // a run: the ulp exponent of its binade; else one of the codes above
};

// Block-wide exclusive scan of ints (kThreads threads); the total in *tot, in every thread.
__device__ inline int32_t block_excl_int(int32_t v, int32_t* tot) {
  __shared__ int32_t ws[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = v;
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t u = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += u;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t y = ws[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, y, d);
      if (lane >= d) y += u;
    }
    ws[lane] = y;
  }
  __syncthreads();
  *tot = ws[kThreads / 32 - 1];
  const int32_t r = (w ? ws[w - 1] : 0) + x - v;
  __syncthreads();
  return r;
}

// Block-wide exclusive scan of doubles (any rounding order: an approximation).
__device__ inline double block_excl_approx(double v) {
  __shared__ double ws[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double x = v;
  for (int d = 1; d < 32; d <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += u;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    double y = ws[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const double u = __shfl_up_sync(0xffffffffu, y, d);
      if (lane >= d) y += u;
    }
    ws[lane] = y;
  }
  __syncthreads();
  const double r = (w ? ws[w - 1] : 0.0) + (x - v);
  __syncthreads();
  return r;
}

// Block-wide sum of doubles (any rounding order: an approximation), in every thread.
__device__ inline double block_sum_approx(double v) {
  __shared__ double ws[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double y = ws[lane];
  for (int d = 16; d > 0; d >>= 1) y += __shfl_xor_sync(0xffffffffu, y, d);
  __syncthreads();
  return y;
}

// A term's segment code from the approximate sums before (pe) and after (pi) it, by integer
// tests on their bits (the FP64 pipe is the scarce one): a run code when both are normal, in
// one binade, and at least about 1.5e-8 of it inside (mantissa fractions above kLowGuard and
// below the top by kHighGuard, in ulps of 2^52), else a single.
constexpr uint64_t kMant = (uint64_t(1) << 52) - 1;
constexpr uint64_t kLowGuard = uint64_t(1) << 26;   // 1.5e-8 of the binade's bottom
constexpr uint64_t kHighGuard = uint64_t(1) << 27;  // 1.5e-8 of its top
__device__ __forceinline__ int32_t seg_code(double t, double pe, double pi) {
  const uint64_t bt = uint64_t(__double_as_longlong(t));
  const uint64_t be = uint64_t(__double_as_longlong(pe)), bi = uint64_t(__double_as_longlong(pi));
  if ((bt | bi) == 0) return kSkipCode;  // (+0 + +0: zeros before the first nonzero term)
  const uint64_t ee = be >> 52, ei = bi >> 52;  // (a sign bit makes these large)
  if (ee == 0 || ee >= 0x7fe || ei != ee) return kSingleCode;
  if ((be & kMant) < kLowGuard || (bi & kMant) > kMant - kHighGuard) return kSingleCode;
  return int32_t(ee) - 1075;
}

// segmented scan element: f = a segment starts inside, v = the pairs since the last start,
// st = the last start's index
struct SegScan {
  int32_t f;
  Pair v;
  int64_t st;
};

__device__ __forceinline__ SegScan seg_op(const SegScan& x, const SegScan& y) {
  return SegScan{x.f | y.f, y.f ? y.v : compose(x.v, y.v), y.f ? y.st : x.st};
}

__device__ __forceinline__ SegScan shfl_up_seg(const SegScan& x, int d) {
  SegScan r;
  r.f = __shfl_up_sync(0xffffffffu, x.f, d);
  r.v.d0 = __shfl_up_sync(0xffffffffu, x.v.d0, d);
  r.v.d1 = __shfl_up_sync(0xffffffffu, x.v.d1, d);
  r.st = __shfl_up_sync(0xffffffffu, x.st, d);
  return r;
}

__device__ __forceinline__ Pair seg_pair(double t, int32_t code) {
  return code < kSkipCode ? term_pair(t, code) : Pair{0, 0};
}

// The segments of terms [a, b) (b - a <= kTile; before: the approximate sum of the terms
// before a), in order, to out[0, kTileSegs); returns their count in every thread (more than
// kTileSegs: only counted), and the tile's approximate sum in *tile_total when given.
template <class Term>
__device__ int32_t build_segments(int64_t a, int64_t b, double before, Term term, Seg* out,
                                  double* tile_total = nullptr) {
  __shared__ int32_t first_code[kThreads / 32], last_code[kThreads / 32];
  __shared__ SegScan wsc[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t base = a + int64_t(threadIdx.x) * kItems;
  double t[kItems];
  double own = 0.0;
#pragma unroll
  for (int it = 0; it < kItems; ++it) {
    t[it] = base + it < b ? term(base + it) : 0.0;
    own += t[it];
  }
  double pe = before + block_excl_approx(own);
  if (tile_total) *tile_total = block_sum_approx(own);
  int32_t code[kItems];
#pragma unroll
  for (int it = 0; it < kItems; ++it) {
    const double pi = pe + t[it];
    code[it] = seg_code(t[it], pe, pi);
    pe = pi;
  }
  // neighbours' codes across thread and warp edges
  int32_t prev = __shfl_up_sync(0xffffffffu, code[kItems - 1], 1);
  int32_t next = __shfl_down_sync(0xffffffffu, code[0], 1);
  if (lane == 0) first_code[w] = code[0];
  if (lane == 31) last_code[w] = code[kItems - 1];
  __syncthreads();
  if (lane == 0) prev = w ? last_code[w - 1] : kSingleCode;
  if (lane == 31) next = w + 1 < kThreads / 32 ? first_code[w + 1] : kSingleCode;
  // start / end bits of the valid items
  unsigned start = 0, end = 0;
#pragma unroll
  for (int it = 0; it < kItems; ++it) {
    const int64_t k = base + it;
    if (k >= b) break;
    const int32_t p = it ? code[it - 1] : prev, n = it + 1 < kItems ? code[it + 1] : next;
    const int32_t c = code[it];
    if (k == a || c == kSingleCode || p == kSingleCode || c != p) start |= 1u << it;
    if (k == b - 1 || n == kSingleCode || c == kSingleCode || n != c) end |= 1u << it;
  }
  // segmented scan of the pairs: this thread's aggregate, then the block's exclusive prefix
  SegScan agg{0, Pair{0, 0}, -1};
#pragma unroll
  for (int it = 0; it < kItems; ++it) {
    if (base + it >= b) break;
    const SegScan e{int32_t((start >> it) & 1u), seg_pair(t[it], code[it]), base + it};
    agg = seg_op(agg, e);
  }
  SegScan incl = agg;
  for (int d = 1; d < 32; d <<= 1) {
    const SegScan u = shfl_up_seg(incl, d);
    if (lane >= d) incl = seg_op(u, incl);
  }
  SegScan ex = shfl_up_seg(incl, 1);
  if (lane == 0) ex = SegScan{0, Pair{0, 0}, -1};
  if (lane == 31) wsc[w] = incl;
  __syncthreads();
  if (w == 0) {
    SegScan y = wsc[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const SegScan u = shfl_up_seg(y, d);
      if (lane >= d) y = seg_op(u, y);
    }
    wsc[lane] = y;
  }
  __syncthreads();
  if (w) ex = seg_op(wsc[w - 1], ex);
  // record slots
  int32_t total;
  int32_t idx = block_excl_int(__popc(end), &total);
  if (total <= kTileSegs) {
    SegScan run = ex;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
      const int64_t k = base + it;
      if (k >= b) break;
      const SegScan e{int32_t((start >> it) & 1u), seg_pair(t[it], code[it]), k};
      run = seg_op(run, e);
      if ((end >> it) & 1u) {
        Seg r;
        r.pair = run.v;
        r.t = t[it];
        r.first = run.st;
        r.count = int32_t(k - run.st + 1);
        r.code = code[it];
        out[idx++] = r;
      }
    }
  }
  return total;
}

// The sequential sum from s0 over the segments of tiles tile0 + [0, ntile): tile tile0 + i's
// cnt[i] records at rec + i kTileSegs, or, for cnt[i] < 0, its terms term by term. Every thread
// gets the result (after a non-finite partial sum: the final one, all later terms looked at).
constexpr int kWalkBatch = 512;
template <class Term>
__device__ double walk_segments(double s0, int32_t tile0, int32_t ntile, const int32_t* cnt, const Seg* rec,
                                int64_t m, Term term) {
  __shared__ Seg batch[kWalkBatch];
  __shared__ int32_t woff[kThreads + 1];
  __shared__ double s_sh;
  __shared__ int32_t j_sh, act_sh;
  __shared__ int64_t fa_sh, fb_sh;
  if (threadIdx.x == 0) {
    s_sh = s0;
    act_sh = 0;
  }
  __syncthreads();
  bool nonfinite = false;
  for (int32_t c0 = 0; c0 < ntile && !nonfinite; c0 += kThreads) {
    const int32_t nw = ntile - c0 < kThreads ? ntile - c0 : kThreads;
    const int32_t cc = int32_t(threadIdx.x) < nw ? cnt[c0 + threadIdx.x] : 0;
    int32_t tot;
    const int32_t ex = block_excl_int(cc < 0 ? 1 : cc, &tot);
    woff[threadIdx.x] = ex;
    if (threadIdx.x == 0) woff[nw] = tot;
    __syncthreads();
    for (int32_t g0 = 0; g0 < tot && !nonfinite; g0 += kWalkBatch) {
      const int32_t nb = tot - g0 < kWalkBatch ? tot - g0 : kWalkBatch;
      if (int32_t(threadIdx.x) < nb) {
        const int32_t g = g0 + int32_t(threadIdx.x);
        int lo = 0, hi = nw - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (woff[mid] <= g) lo = mid;
          else hi = mid - 1;
        }
        const int32_t c = c0 + lo;
        const int32_t n = cnt[c];
        if (n < 0) {
          const int64_t ta = int64_t(tile0 + c) * kTile, tb = ta + kTile < m ? ta + kTile : m;
          batch[threadIdx.x] = Seg{Pair{0, 0}, 0.0, ta, int32_t(tb - ta), kRangeCode};
        } else {
          batch[threadIdx.x] = rec[int64_t(c) * kTileSegs + (g - woff[lo])];
        }
      }
      __syncthreads();
      int32_t j = 0;
      while (true) {
        if (threadIdx.x == 0) {
          double s = s_sh;
          int act = 0;
          int64_t fa = 0, fb = 0;
          for (; j < nb; ++j) {
            const Seg& r = batch[j];
            if (r.code == kSkipCode) continue;
            if (r.code == kSingleCode) {
              s = __dadd_rn(s, r.t);
              if (!(s < INFINITY)) {  // inf or NaN
                act = 2;
                fa = r.first + 1;
                ++j;
                break;
              }
              continue;
            }
            if (r.code != kRangeCode && s > 0.0) {
              int64_t S;
              int ue;
              split(s, &S, &ue);
              if (ue == r.code) {
                const int64_t S2 = sat(S, pick(r.pair, S));
                if (S2 < kTop) {
                  s = join(S2, ue);
                  continue;
                }
              }
            }
            act = 1;
            fa = r.first;
            fb = r.first + r.count;
            ++j;
            break;
          }
          s_sh = s;
          act_sh = act;
          j_sh = j;
          fa_sh = fa;
          fb_sh = fb;
        }
        __syncthreads();
        const int act = act_sh;
        j = j_sh;
        if (act == 0) break;
        if (act == 2) {
          nonfinite = true;
          break;
        }
        const double s1 = sequential_sum_from(s_sh, fa_sh, fb_sh, term);
        __syncthreads();
        if (threadIdx.x == 0) s_sh = s1;
        __syncthreads();
        if (!(s1 < INFINITY)) {
          // (sequential_sum_from already looked at its range's later terms)
          nonfinite = true;
          if (threadIdx.x == 0) fa_sh = fb_sh;
          __syncthreads();
          break;
        }
      }
      __syncthreads();
    }
  }
  double s = s_sh;
  if (nonfinite && s == s) {
    // inf: NaN if any later term is NaN
    const int64_t from = fa_sh;
    int nan = 0;
    for (int64_t k = from + threadIdx.x; k < m; k += kThreads) {
      const double x = term(k);
      if (x != x) nan = 1;
    }
    if (__syncthreads_or(nan)) s = __longlong_as_double(0x7ff8000000000000LL);
  }
  __syncthreads();
  return s;
}

}  // namespace exact
}  // namespace svxg
