// exact_sum.cuh - the sequential double sum s = ((0 + t_0) + t_1) + ... of nonnegative terms,
// computed in parallel with the very same result bits.
//
// The reference sums some nonnegative sequences one term after another (the power iteration's
// norm, core/src/solve/amg.cpp:267-268; id_scale, core/src/stress/stress.cpp:112-122). A
// parallel tree would round differently, so the device reproduces the sequential rounding:
// while the running sum s stays inside one binade [2^e, 2^(e+1)) (ulp U fixed), s is an
// integer S times U and every addition fl(s + t) is S + round(t / U), the rounding of t / U to an
// integer with ties broken to the even result - i.e. by the parity of S. Each term is therefore
// a pair of integer increments (delta if S is even, delta if S is odd), and pairs compose
// associatively (the second's choice keyed by the parity after the first): a block-wide scan of
// pairs gives the running S at every position. The first position where S would leave the
// binade (S >= 2^53; a term at least 2^(e+1), infinite or NaN also counts) is found by a block
// minimum; there the addition is done by the hardware (IEEE add), the binade changes and the
// scan resumes. The sum crosses at most a few dozen binades, so the work stays O(n).
// Integer arithmetic only, apart from those crossing additions.
#pragma once

#include <cstdint>

namespace svxg {
namespace exact {

constexpr int kThreads = 1024;
constexpr int kItems = 8;
constexpr int kQuietRounds = 4;  // warp rounds without a crossing before block rounds resume
constexpr int64_t kWarpSumMax = 4096;  // sums of at most this many terms go to one warp
constexpr int64_t kCap = int64_t(1) << 54;  // saturation: past any binade's room

struct Pair {
  int64_t d0, d1;  // increments (in ulps) from an even / odd S
};

__device__ __forceinline__ int64_t sat(int64_t a, int64_t b) {
  const int64_t s = a + b;
  return s > kCap ? kCap : s;
}

// x then y
__device__ __forceinline__ Pair compose(Pair x, Pair y) {
  Pair r;
  r.d0 = sat(x.d0, (x.d0 & 1) ? y.d1 : y.d0);
  r.d1 = sat(x.d1, (x.d1 & 1) ? y.d0 : y.d1);
  return r;
}

// the increment pair of adding t (>= 0) to s = S U with U = 2^uexp; kCap marks a crossing term
__device__ __forceinline__ Pair term_pair(double t, int uexp) {
  const uint64_t bits = uint64_t(__double_as_longlong(t));
  const int E = int((bits >> 52) & 0x7ff);
  if (E == 0x7ff || (bits >> 63)) return {kCap, kCap};  // inf / NaN (/ negative: not expected)
  uint64_t m;
  int et;
  if (E == 0) {
    m = bits & ((uint64_t(1) << 52) - 1);
    et = -1074;
  } else {
    m = (bits & ((uint64_t(1) << 52) - 1)) | (uint64_t(1) << 52);
    et = E - 1075;
  }
  if (m == 0) return {0, 0};
  const int sh = et - uexp;  // t / U = m 2^sh
  if (sh >= 0) {
    if (sh > 1) return {kCap, kCap};  // t >= 2^(e+1): a crossing (m >= 2^52 when normal)
    const uint64_t a = m << sh;
    if (a >= (uint64_t(1) << 53)) return {kCap, kCap};
    return {int64_t(a), int64_t(a)};
  }
  const int r = -sh;
  if (r > 60) return {0, 0};  // t / U < 2^-7: rounds to 0 whatever the parity
  const uint64_t I = m >> r;
  const uint64_t rem = m & ((uint64_t(1) << r) - 1);
  const uint64_t half = uint64_t(1) << (r - 1);
  if (rem < half) return {int64_t(I), int64_t(I)};
  if (rem > half) return {int64_t(I + 1), int64_t(I + 1)};
  // a tie: the even result
  const int64_t Ii = int64_t(I);
  return {Ii + ((Ii & 1) ? 1 : 0), Ii + ((Ii & 1) ? 0 : 1)};
}

// s = S 2^uexp, S < 2^53 (normal or subnormal)
__device__ __forceinline__ void split(double s, int64_t* S, int* uexp) {
  const uint64_t bits = uint64_t(__double_as_longlong(s));
  const int E = int((bits >> 52) & 0x7ff);
  if (E == 0) {
    *S = int64_t(bits & ((uint64_t(1) << 52) - 1));
    *uexp = -1074;
  } else {
    *S = int64_t((bits & ((uint64_t(1) << 52) - 1)) | (uint64_t(1) << 52));
    *uexp = E - 1075;
  }
}

__device__ __forceinline__ double join(int64_t S, int uexp) {
  // S < 2^53; uexp = -1074 with S < 2^52 is subnormal
  if (S < (int64_t(1) << 52)) {
    // only reachable for uexp = -1074 (a normal start keeps S >= 2^52)
    return __longlong_as_double((long long)S);
  }
  const uint64_t E = uint64_t(uexp + 1075);
  return __longlong_as_double((long long)((E << 52) | (uint64_t(S) & ((uint64_t(1) << 52) - 1))));
}

__device__ __forceinline__ Pair shfl_up_pair(Pair v, int d) {
  Pair u;
  u.d0 = __shfl_up_sync(0xffffffffu, v.d0, d);
  u.d1 = __shfl_up_sync(0xffffffffu, v.d1, d);
  return u;
}

// inclusive scan of the warp's pairs (whole warp)
__device__ __forceinline__ Pair warp_scan(Pair v) {
  const int lane = threadIdx.x & 31;
  for (int d = 1; d < 32; d <<= 1) {
    const Pair u = shfl_up_pair(v, d);
    if (lane >= d) v = compose(u, v);
  }
  return v;
}

// Block-wide exclusive scan of pairs (kThreads threads): warps scan by shuffles, then the warps'
// totals; returns the exclusive prefix of this thread's pair and the block total in *tot.
__device__ inline Pair block_scan(Pair v, Pair* tot) {
  __shared__ Pair wsum[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const Pair incl = warp_scan(v);
  Pair ex_w = shfl_up_pair(incl, 1);
  if (lane == 0) ex_w = Pair{0, 0};
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const Pair x = warp_scan(wsum[lane]);  // (kThreads / 32 == 32 warps)
    wsum[lane] = x;
  }
  __syncthreads();
  const Pair before = w ? wsum[w - 1] : Pair{0, 0};
  *tot = wsum[kThreads / 32 - 1];
  __syncthreads();
  return compose(before, ex_w);
}

__device__ __forceinline__ int64_t pick(Pair p, int64_t S) { return (S & 1) ? p.d1 : p.d0; }

// The sequential sum s0 + term(a) + ... + term(n - 1), added one by one from s0 (>= 0), with
// term(k) >= 0; one block of kThreads. Term: a callable (int64_t k) -> double. Every thread gets
// the result.
template <class Term>
__device__ inline double sequential_sum_from(double s0, int64_t a, int64_t n, Term term) {
  __shared__ double s_sh;
  __shared__ int64_t p_sh;
  __shared__ int64_t first_sh;
  __shared__ int quiet_sh;  // warp rounds in a row without a crossing
  if (threadIdx.x == 0) {
    s_sh = s0;
    p_sh = a;
    quiet_sh = 0;
  }
  __syncthreads();
  constexpr int64_t kTile = int64_t(kThreads) * kItems;
  while (true) {
    const int64_t p = p_sh;
    const double s = s_sh;
    const bool warp_round = quiet_sh < kQuietRounds;
    __syncthreads();
    if (p >= n) break;
    const uint64_t sbits = uint64_t(__double_as_longlong(s));
    if (((sbits >> 52) & 0x7ff) == 0x7ff) {
      // s is inf or NaN: NaN if any later term is NaN, else s
      __shared__ int nan_sh;
      if (threadIdx.x == 0) nan_sh = 0;
      __syncthreads();
      for (int64_t k = p + threadIdx.x; k < n; k += kThreads)
        if (term(k) != term(k)) nan_sh = 1;
      __syncthreads();
      const double r = (nan_sh && s == s) ? __longlong_as_double(0x7ff8000000000000LL) : s;
      __syncthreads();
      return r;
    }
    if (s == 0.0) {
      // leading zeros leave s at 0; the first nonzero term becomes s exactly
      if (threadIdx.x == 0) first_sh = n;
      __syncthreads();
      for (int64_t b = p; b < n && first_sh == n; b += kTile) {
        for (int it = 0; it < kItems; ++it) {
          const int64_t k = b + int64_t(it) * kThreads + threadIdx.x;
          if (k < n) {
            const double t = term(k);
            if (!(t == 0.0)) atomicMin((unsigned long long*)&first_sh, (unsigned long long)k);
          }
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        if (first_sh < n) {
          s_sh = 0.0 + term(first_sh);
          p_sh = first_sh + 1;
        } else {
          p_sh = n;
        }
      }
      __syncthreads();
      continue;
    }
    int64_t S;
    int uexp;
    split(s, &S, &uexp);
    if (warp_round) {
      // While crossings come close together (a small running sum: the start, after a crossing),
      // one warp takes 32 terms a round, which costs far less than a block round.
      if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int64_t k = p + lane;
        const double t = k < n ? term(k) : 0.0;
        const Pair pr = k < n ? term_pair(t, uexp) : Pair{0, 0};
        const Pair incl = warp_scan(pr);
        Pair ex = shfl_up_pair(incl, 1);
        if (lane == 0) ex = Pair{0, 0};
        const int64_t run = sat(S, pick(ex, S));
        const bool cross = k < n && sat(run, pick(pr, run)) >= (int64_t(1) << 53);
        const unsigned m = __ballot_sync(0xffffffffu, cross);
        if (m == 0) {
          Pair tot;
          tot.d0 = __shfl_sync(0xffffffffu, incl.d0, 31);
          tot.d1 = __shfl_sync(0xffffffffu, incl.d1, 31);
          if (lane == 0) {
            s_sh = join(sat(S, pick(tot, S)), uexp);
            p_sh = p + 32 < n ? p + 32 : n;
            quiet_sh = quiet_sh + 1;
          }
        } else {
          if (lane == __ffs(m) - 1) {
            s_sh = __dadd_rn(join(run, uexp), t);
            p_sh = k + 1;
          }
          if (lane == 0) quiet_sh = 0;
        }
      }
      __syncthreads();
      continue;
    }
    // this thread's kItems consecutive terms
    const int64_t base = p + int64_t(threadIdx.x) * kItems;
    Pair loc[kItems];
    Pair acc{0, 0};
    for (int it = 0; it < kItems; ++it) {
      const int64_t k = base + it;
      loc[it] = k < n ? term_pair(term(k), uexp) : Pair{0, 0};
      acc = compose(acc, loc[it]);
    }
    Pair tot;
    const Pair ex = block_scan(acc, &tot);
    // the first position where S leaves the binade
    if (threadIdx.x == 0) first_sh = INT64_MAX;
    __syncthreads();
    {
      int64_t run = sat(S, pick(ex, S));
      for (int it = 0; it < kItems; ++it) {
        const int64_t k = base + it;
        if (k >= n) break;
        const int64_t nxt = sat(run, pick(loc[it], run));
        if (nxt >= (int64_t(1) << 53)) {
          atomicMin((unsigned long long*)&first_sh, (unsigned long long)k);
          break;
        }
        run = nxt;
      }
    }
    __syncthreads();
    const int64_t firstx = first_sh;
    const int64_t end = p + kTile < n ? p + kTile : n;
    if (firstx == INT64_MAX) {
      if (threadIdx.x == 0) {
        s_sh = join(sat(S, pick(tot, S)), uexp);
        p_sh = end;
      }
    } else {
      // S just before the crossing: the thread that owns it replays its prefix
      const int64_t owner = (firstx - p) / kItems;
      if (int64_t(threadIdx.x) == owner) {
        int64_t run = sat(S, pick(ex, S));
        for (int64_t k = base; k < firstx; ++k) run = sat(run, pick(loc[k - base], run));
        const double before = join(run, uexp);
        s_sh = __dadd_rn(before, term(firstx));
        p_sh = firstx + 1;
        quiet_sh = 0;  // (crossings come in runs: warp rounds until it is quiet again)
      }
    }
    __syncthreads();
  }
  const double r = s_sh;
  __syncthreads();
  return r;
}

// The same by one warp (the only threads that call it), for short sequences: rounds of 32 terms
// with no block-wide barrier. Every lane gets the result.
template <class Term>
__device__ inline double warp_sequential_sum_from(double s, int64_t p, int64_t n, Term term) {
  const int lane = threadIdx.x & 31;
  while (p < n) {
    const uint64_t sbits = uint64_t(__double_as_longlong(s));
    if (((sbits >> 52) & 0x7ff) == 0x7ff) {
      // s is inf or NaN: NaN if any later term is NaN, else s
      bool nan = false;
      for (int64_t k = p + lane; k < n; k += 32) nan |= term(k) != term(k);
      const bool any = __any_sync(0xffffffffu, nan);
      return (any && s == s) ? __longlong_as_double(0x7ff8000000000000LL) : s;
    }
    if (s == 0.0) {
      // leading zeros leave s at 0; the first nonzero term becomes s exactly
      const int64_t k = p + lane;
      const double t = k < n ? term(k) : 0.0;
      const unsigned m = __ballot_sync(0xffffffffu, k < n && !(t == 0.0));
      if (m == 0) {
        p = p + 32;
        continue;
      }
      const int f = __ffs(m) - 1;
      s = 0.0 + __shfl_sync(0xffffffffu, t, f);
      p = p + f + 1;
      continue;
    }
    int64_t S;
    int uexp;
    split(s, &S, &uexp);
    const int64_t k = p + lane;
    const double t = k < n ? term(k) : 0.0;
    const Pair pr = k < n ? term_pair(t, uexp) : Pair{0, 0};
    const Pair incl = warp_scan(pr);
    Pair ex = shfl_up_pair(incl, 1);
    if (lane == 0) ex = Pair{0, 0};
    const int64_t run = sat(S, pick(ex, S));
    const bool cross = k < n && sat(run, pick(pr, run)) >= (int64_t(1) << 53);
    const unsigned m = __ballot_sync(0xffffffffu, cross);
    if (m == 0) {
      Pair tot;
      tot.d0 = __shfl_sync(0xffffffffu, incl.d0, 31);
      tot.d1 = __shfl_sync(0xffffffffu, incl.d1, 31);
      s = join(sat(S, pick(tot, S)), uexp);
      p = p + 32;
    } else {
      const int f = __ffs(m) - 1;
      const double before = __shfl_sync(0xffffffffu, join(run, uexp), f);
      s = __dadd_rn(before, __shfl_sync(0xffffffffu, t, f));
      p = p + f + 1;
    }
  }
  return s;
}

// The sequential sum of term(k) for k in [0, n) from 0.
template <class Term>
__device__ inline double sequential_sum(int64_t n, Term term) {
  return sequential_sum_from(0.0, 0, n, term);
}

}  // namespace exact
}  // namespace svxg
