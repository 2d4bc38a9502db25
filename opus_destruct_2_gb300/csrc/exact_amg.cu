// exact_amg.cu - the aggregation multigrid built on the device, value for value the reference's
// hierarchy (Amg::build / finalize / estimate_lmax / coarsen / factor_coarsest,
// core/src/solve/amg.cpp:228-578). Compiled with -fmad=false: every sum runs in the reference's
// order with separate multiplies and adds, divisions and square roots IEEE-rounded.
//
// fast_amg.cu compiles this file a second time with SVXG_FAST_SETUP defined and without
// -fmad=false (build_hierarchy_fast, the mixed-precision policy's setup): the same algorithm and
// summation orders with multiplies and adds contracted into FMAs, and the power iteration's norm
// as a fixed-order tree sum instead of the sequential sum - deterministic, within rounding of the
// reference's values, at about half the FP64 instructions (this part issues FP64 at two lanes a
// clock per SM, and the bit-exact products are bound by that). Its aggregates can differ from
// the reference's where a strength test sits within rounding of its threshold.
//
// The reference's aggregation is sequential (amg.cpp:339-349: node i becomes a root when it is
// not aggregated and none of its strong neighbours is, then claims them). Its roots are the
// lexicographically first independent set of the conflict graph "N[r] and N[i] meet"
// (N[x] = x and its strong neighbours by row x): i is a root iff no lower root conflicts with it.
// The device decides that set in rounds, each deciding every node whose lower conflicting nodes
// are all decided:
//   claim:  every undecided node i writes min(i) into claim[x] for x in N[i];
//   decide: i becomes a non-root if some x in N[i] is covered by an earlier root, a root if it
//           holds every claim in N[i] (then no undecided lower node conflicts with it);
//   cover:  each new root covers N[r] (disjoint from other roots' by construction).
// The smallest undecided node always decides, so the rounds end; the result is the reference's
// root set exactly, and the aggregate ids follow as the roots' ranks. Passes 2 and 3
// (amg.cpp:351-384) are per-node and scan steps. Sums whose order matters (coarse positions,
// prolongation rows, Galerkin products, the power iteration's norm) run in the reference's order.
#include <algorithm>
#include <climits>
#include <cmath>

#include "blk6.cuh"
#include "exact_runs.cuh"
#include "exact_sum.cuh"
#include "problem.cuh"
#include "spmv_row.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;
inline unsigned nblk(int64_t n, int t = kT) { return unsigned(std::max<int64_t>(1, (n + t - 1) / t)); }

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

template <class T>
struct Tmp {
  T* p = nullptr;
  cudaStream_t s;
  explicit Tmp(cudaStream_t st) : s(st) {}
  int alloc(size_t n) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    cudaError_t e = pool_malloc_async(reinterpret_cast<void**>(&p), (n ? n : 1) * sizeof(T), s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(std::string("device allocation: ") + cudaGetErrorString(e));
      p = nullptr;
      return e == cudaErrorMemoryAllocation ? SVXG_ERR_NOMEM : SVXG_ERR_CUDA;
    }
    return SVXG_OK;
  }
  ~Tmp() {
    if (p) cudaFreeAsync(p, s);
  }
};

// ---- finalize (amg.cpp:228-254) --------------------------------------------------------------
__global__ void k_dinv(int32_t n, const int32_t* rowptr, const double* val, double* dinv, int32_t* fail) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double tmp[36];
  if (!inv6_regularised(val + 36 * int64_t(rowptr[i]), tmp)) atomicExch(fail, 1);
  for (int q = 0; q < 36; ++q) dinv[36 * int64_t(i) + q] = tmp[q];
}

// ---- estimate_lmax (amg.cpp:256-275) ------------------------------------------------------------
__global__ void k_lmax_init(int64_t m, double* v) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m) v[k] = 1.0 + 0.001 * (double)(k % 7);
}

// entry t = 6 i + r of A x in Bsr6::apply's order (blocks in row order)
__device__ __forceinline__ double spmv_exact_entry(int64_t t, const int32_t* rowptr, const int32_t* col,
                                                   const double* val, const double* x) {
  const int32_t i = int32_t(t / 6);
  const int r = int(t % 6);
  double yr = 0.0;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const double* m = val + 36 * int64_t(k) + 6 * r;
    const double* xv = x + 6 * int64_t(col[k]);
    yr += m[0] * xv[0] + m[1] * xv[1] + m[2] * xv[2] + m[3] * xv[3] + m[4] * xv[4] + m[5] * xv[5];
  }
  return yr;
}

// state: [0] = lam, [1] = nv, [2] = stopped
// Power iteration step: v' = D^-1 (A v) with one thread per entry (the node's six entries of A v
// meet in shared memory, each in Bsr6::apply's order, then mv6's row), then the exact norm with
// the step's lam / stop / scaling (launch_norm).
constexpr int kApplyNodes = 32;  // nodes per block: 192 threads
__global__ void __launch_bounds__(6 * kApplyNodes) k_lmax_apply(int32_t n, const int32_t* rowptr, const int32_t* col,
                                                              const double* val, const double* dinv, const double* v,
                                                              double* w, const double* state) {
  __shared__ double y[6 * kApplyNodes];
  if (state[2] != 0.0) return;
  const int64_t t = int64_t(blockIdx.x) * (6 * kApplyNodes) + threadIdx.x;
  const bool ok = t < 6 * int64_t(n);
  y[threadIdx.x] = ok ? spmv_exact_entry(t, rowptr, col, val, v) : 0.0;
  __syncthreads();
  if (!ok) return;
  const int32_t i = int32_t(t / 6);
  const int r = int(t % 6);
  const double* x = y + 6 * (threadIdx.x / 6);
  const double* m = dinv + 36 * int64_t(i) + 6 * r;
  w[t] = m[0] * x[0] + m[1] * x[1] + m[2] * x[2] + m[3] * x[3] + m[4] * x[4] + m[5] * x[5];
}

// The same step for shorter levels with longer rows, a warp per node: the six-term products of
// the row's blocks (entry, block items over the lanes, chunks of kApplyChunk blocks) first, then
// lanes 0-5 add them in block order - the same sums as spmv_exact_entry - and D^-1 (A v).
constexpr int kApplyChunk = 48;
constexpr int kApplyWarps = 4;
constexpr int32_t kApplyRowsMax = 16384;  // levels up to this many nodes take the warp-per-node form
__global__ void __launch_bounds__(32 * kApplyWarps) k_lmax_apply_rows(int32_t n, const int32_t* rowptr,
                                                                      const int32_t* col, const double* val,
                                                                      const double* dinv, const double* v, double* w,
                                                                      const double* state) {
  __shared__ double d_sh[kApplyWarps][6 * kApplyChunk];
  __shared__ double y_sh[kApplyWarps][6];
  if (state[2] != 0.0) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t i = int32_t(blockIdx.x) * kApplyWarps + wid;
  if (i >= n) return;
#ifdef SVXG_FAST_SETUP
  (void)d_sh;
  const double yr = warp_row_product<double, double, double>(rowptr[i], rowptr[i + 1], col, val, v);
#else
  double yr = 0.0;
  for (int32_t kb = rowptr[i]; kb < rowptr[i + 1]; kb += kApplyChunk) {
    const int32_t nk = rowptr[i + 1] - kb < kApplyChunk ? rowptr[i + 1] - kb : kApplyChunk;
    for (int32_t it = lane; it < 6 * nk; it += 32) {
      const int32_t kl = it / 6;
      const int r = it - 6 * kl;
      const double* m = val + 36 * int64_t(kb + kl) + 6 * r;
      const double* xv = v + 6 * int64_t(col[kb + kl]);
      d_sh[wid][it] = m[0] * xv[0] + m[1] * xv[1] + m[2] * xv[2] + m[3] * xv[3] + m[4] * xv[4] + m[5] * xv[5];
    }
    __syncwarp();
    if (lane < 6)
      for (int32_t kl = 0; kl < nk; ++kl) yr += d_sh[wid][6 * kl + lane];
    __syncwarp();
  }
#endif
  if (lane < 6) y_sh[wid][lane] = yr;
  __syncwarp();
  if (lane < 6) {
    const double* x = y_sh[wid];
    const double* m = dinv + 36 * int64_t(i) + 6 * lane;
    w[6 * int64_t(i) + lane] = m[0] * x[0] + m[1] * x[1] + m[2] * x[2] + m[3] * x[3] + m[4] * x[4] + m[5] * x[5];
  }
}

// The exact norm: sqrt of the sequential sum of w_k^2 (amg.cpp:267-268: the reference's
// v[i] * v[i], one rounding each) by predicted binade runs (exact_runs.cuh). Vectors of at most
// exact::kTile terms take one block (k_norm_small, with the scaling v = w / nv); longer ones a
// tile per block: approximate tile sums, each tile's segments, one block's ordered walk, then
// the scaling.
struct SqTerm {
  const double* w;
  __device__ __forceinline__ double operator()(int64_t k) const {
    const double x = w[k];
    return x * x;
  }
};

// state[0] = lam <- nv, state[1] = nv; a zero or non-finite norm stops the iteration
__device__ __forceinline__ void set_norm(double* state, double nv) {
  state[1] = nv;
  if (!(nv > 0)) state[2] = 1.0;
  else state[0] = nv;
}

__global__ void __launch_bounds__(exact::kThreads) k_norm_small(int64_t m, const double* w, double* v,
                                                               exact::Seg* rec, int32_t* cnt, double* state) {
  __shared__ double nv_sh;
  if (state[2] != 0.0) return;
  const int32_t n = exact::build_segments(0, m, 0.0, SqTerm{w}, rec);
  if (threadIdx.x == 0) cnt[0] = n > exact::kTileSegs ? -1 : n;
  __syncthreads();
  const double s = exact::walk_segments(0.0, 0, 1, cnt, rec, m, SqTerm{w});
  if (threadIdx.x == 0) {
    nv_sh = sqrt(s);
    set_norm(state, nv_sh);
  }
  __syncthreads();
  const double nv = nv_sh;
  if (!v || !(nv > 0)) return;
  for (int64_t k = threadIdx.x; k < m; k += exact::kThreads) v[k] = w[k] / nv;
}

// a vector of a few tiles in one block, tile after tile: each tile's segments, then the walk over
// them from the running sum (a launch instead of four: small requests are launch-bound)
constexpr int64_t kNormLoopMax = 2 * exact::kTile;  // (beyond two tiles the per-tile launches are faster)
__global__ void __launch_bounds__(exact::kThreads) k_norm_loop(int64_t m, const double* w, double* v,
                                                              exact::Seg* rec, int32_t* cnt, double* state) {
  __shared__ double nv_sh;
  if (state[2] != 0.0) return;
  double s = 0.0, before = 0.0;
  const int32_t ntile = int32_t((m + exact::kTile - 1) / exact::kTile);
  for (int32_t c = 0; c < ntile; ++c) {
    const int64_t a = int64_t(c) * exact::kTile, b = a + exact::kTile < m ? a + exact::kTile : m;
    double tile = 0.0;
    const int32_t n = exact::build_segments(a, b, before, SqTerm{w}, rec, &tile);
    if (threadIdx.x == 0) cnt[0] = n > exact::kTileSegs ? -1 : n;
    __syncthreads();
    s = exact::walk_segments(s, c, 1, cnt, rec, m, SqTerm{w});
    if (!(s < INFINITY)) break;  // (the walk has looked at every later term)
    before += tile;
  }
  if (threadIdx.x == 0) {
    nv_sh = sqrt(s);
    set_norm(state, nv_sh);
  }
  __syncthreads();
  const double nv = nv_sh;
  if (!v || !(nv > 0)) return;
  for (int64_t k = threadIdx.x; k < m; k += exact::kThreads) v[k] = w[k] / nv;
}

// the same terms read through L2 (a block reading other blocks' writes of the same launch)
struct SqTermCG {
  const double* w;
  __device__ __forceinline__ double operator()(int64_t k) const {
    const double x = __ldcg(w + k);
    return x * x;
  }
};

// A power iteration step of a level of at most exact::kTile unknowns in one launch: the warps
// apply D^-1 A v a node each (k_lmax_apply_rows' sums), and the last block to finish takes the
// exact norm and the scaling (k_norm_small's) - one launch a step instead of two, for the small
// problems whose setup is bound by launches.
constexpr int kStepChunk = 12;  // (blocks of a row a warp takes per round: fewer dependent round trips on long coarse rows)
__global__ void __launch_bounds__(exact::kThreads) k_lmax_step_small(int32_t n, const int32_t* rowptr,
                                                                    const int32_t* col, const double* val,
                                                                    const double* dinv, double* v, double* w,
                                                                    exact::Seg* rec, int32_t* cnt, unsigned* counter,
                                                                    double* state) {
  __shared__ double d_sh[exact::kThreads / 32][6 * kStepChunk];
  __shared__ double y_sh[exact::kThreads / 32][6];
  __shared__ bool last;
  __shared__ double nv_sh;
  if (state[2] != 0.0) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t i = int32_t(blockIdx.x) * (exact::kThreads / 32) + wid;
  if (i < n) {
#ifdef SVXG_FAST_SETUP
    // (the fast build: the SpMV's warp-per-row product, its sums in the lanes' order)
    const double yr = warp_row_product<double, double, double>(rowptr[i], rowptr[i + 1], col, val, v);
#else
    double yr = 0.0;
    for (int32_t kb = rowptr[i]; kb < rowptr[i + 1]; kb += kStepChunk) {
      const int32_t nk = rowptr[i + 1] - kb < kStepChunk ? rowptr[i + 1] - kb : kStepChunk;
      for (int32_t it = lane; it < 6 * nk; it += 32) {
        const int32_t kl = it / 6;
        const int r = it - 6 * kl;
        const double* m = val + 36 * int64_t(kb + kl) + 6 * r;
        const double* xv = v + 6 * int64_t(col[kb + kl]);
        d_sh[wid][it] = m[0] * xv[0] + m[1] * xv[1] + m[2] * xv[2] + m[3] * xv[3] + m[4] * xv[4] + m[5] * xv[5];
      }
      __syncwarp();
      if (lane < 6)
        for (int32_t kl = 0; kl < nk; ++kl) yr += d_sh[wid][6 * kl + lane];
      __syncwarp();
    }
#endif
    if (lane < 6) y_sh[wid][lane] = yr;
    __syncwarp();
    if (lane < 6) {
      const double* x = y_sh[wid];
      const double* m = dinv + 36 * int64_t(i) + 6 * lane;
      w[6 * int64_t(i) + lane] = m[0] * x[0] + m[1] * x[1] + m[2] * x[2] + m[3] * x[3] + m[4] * x[4] + m[5] * x[5];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // (every block has read v and written w: the last one may rescale v)
  const int64_t mm = 6 * int64_t(n);
#ifdef SVXG_FAST_SETUP
  (void)rec;
  (void)cnt;
  double part = 0.0;
  for (int64_t k = threadIdx.x; k < mm; k += exact::kThreads) {
    const double x = __ldcg(w + k);
    part += x * x;
  }
  const double sum = exact::block_sum_approx(part);  // (a fixed tree: deterministic)
#else
  const int32_t ns = exact::build_segments(0, mm, 0.0, SqTermCG{w}, rec);
  if (threadIdx.x == 0) cnt[0] = ns > exact::kTileSegs ? -1 : ns;
  __syncthreads();
  const double sum = exact::walk_segments(0.0, 0, 1, cnt, rec, mm, SqTermCG{w});
#endif
  if (threadIdx.x == 0) {
    nv_sh = sqrt(sum);
    set_norm(state, nv_sh);
    *counter = 0u;
  }
  __syncthreads();
  const double nv = nv_sh;
  if (!(nv > 0)) return;
  for (int64_t k = threadIdx.x; k < mm; k += exact::kThreads) v[k] = __ldcg(w + k) / nv;
}

// tile sums (any order: the predictions' approximate prefix)
__global__ void __launch_bounds__(256) k_norm_tile_sum(int64_t m, const double* w, double* tsum, const double* state) {
  __shared__ double sh[256];
  if (state[2] != 0.0) return;
  const int64_t a = int64_t(blockIdx.x) * exact::kTile, b = a + exact::kTile < m ? a + exact::kTile : m;
  double s = 0.0;
  for (int64_t k = a + threadIdx.x; k < b; k += 256) s += w[k] * w[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) tsum[blockIdx.x] = sh[0];
}

// tile c's segments (c = this block)
__global__ void __launch_bounds__(exact::kThreads) k_norm_segments(int64_t m, const double* w, const double* tsum,
                                                                  exact::Seg* rec, int32_t* cnt, const double* state) {
  if (state[2] != 0.0) return;
  const int32_t c = blockIdx.x;
  double before = 0.0;
  for (int32_t j = threadIdx.x; j < c; j += exact::kThreads) before += tsum[j];
  before = exact::block_sum_approx(before);
  const int64_t a = int64_t(c) * exact::kTile, b = a + exact::kTile < m ? a + exact::kTile : m;
  const int32_t n = exact::build_segments(a, b, before, SqTerm{w}, rec + int64_t(c) * exact::kTileSegs);
  if (threadIdx.x == 0) cnt[c] = n > exact::kTileSegs ? -1 : n;
}

__global__ void __launch_bounds__(exact::kThreads) k_norm_walk(int64_t m, int32_t ntile, const double* w,
                                                              const exact::Seg* rec, const int32_t* cnt,
                                                              double* state) {
  if (state[2] != 0.0) return;
  const double s = exact::walk_segments(0.0, 0, ntile, cnt, rec, m, SqTerm{w});
  if (threadIdx.x == 0) set_norm(state, sqrt(s));
}

// v = w / nv for a long vector (after k_norm_walk)
__global__ void k_norm_rescale(int64_t m, const double* w, double* v, const double* state) {
  const double nv = state[1];
  if (!(nv > 0) || state[2] != 0.0) return;
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m) v[k] = w[k] / nv;
}

#ifdef SVXG_FAST_SETUP
// the norm as a fixed-order tree sum: each block's squares summed in a fixed tree, the last block
// to finish adds the blocks' sums in block order and sets state (the grid is fixed by m)
constexpr int kFastNormT = 256;
constexpr int kFastNormBlocks = 1024;
__global__ void __launch_bounds__(kFastNormT) k_norm_fast(int64_t m, const double* w, double* part,
                                                          unsigned* counter, double* state) {
  __shared__ double sh[kFastNormT];
  __shared__ bool last;
  if (state[2] != 0.0) return;
  double s = 0.0;
  for (int64_t k = int64_t(blockIdx.x) * kFastNormT + threadIdx.x; k < m; k += int64_t(gridDim.x) * kFastNormT) {
    const double x = w[k];
    s += x * x;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int d = kFastNormT / 2; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sh[0];
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double t = 0.0;
  for (int b = int(threadIdx.x); b < int(gridDim.x); b += kFastNormT) t += __ldcg(part + b);
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int d = kFastNormT / 2; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    set_norm(state, sqrt(sh[0]));
    *counter = 0u;
  }
}
#endif

// scratch of the exact norm of vectors of m terms
struct NormScratch {
  Tmp<double> tsum;
  Tmp<exact::Seg> rec;
  Tmp<int32_t> cnt;
  int32_t ntile = 0;
  explicit NormScratch(cudaStream_t st) : tsum(st), rec(st), cnt(st) {}
  int alloc(int64_t m) {
    ntile = int32_t(std::max<int64_t>(1, (m + exact::kTile - 1) / exact::kTile));
    TRY(tsum.alloc(size_t(ntile)));
    TRY(rec.alloc(size_t(ntile) * exact::kTileSegs));
    return cnt.alloc(size_t(ntile));
  }
};

// The exact norm of w into state (lam, nv, stopped), and v = w / nv when v is given.
int launch_norm(cudaStream_t st, int64_t m, const double* w, double* v, double* state, NormScratch& S) {
  if (m <= exact::kTile) {
    (k_norm_small<<<1, exact::kThreads, 0, st>>>(m, w, v, S.rec.p, S.cnt.p, state), SVXG_COUNT_LAUNCH());
    return SVXG_OK;
  }
  if (m <= kNormLoopMax) {
    (k_norm_loop<<<1, exact::kThreads, 0, st>>>(m, w, v, S.rec.p, S.cnt.p, state), SVXG_COUNT_LAUNCH());
    return SVXG_OK;
  }
  const unsigned nt = unsigned(S.ntile);
  (k_norm_tile_sum<<<nt, 256, 0, st>>>(m, w, S.tsum.p, state), SVXG_COUNT_LAUNCH());
  (k_norm_segments<<<nt, exact::kThreads, 0, st>>>(m, w, S.tsum.p, S.rec.p, S.cnt.p, state), SVXG_COUNT_LAUNCH());
  (k_norm_walk<<<1, exact::kThreads, 0, st>>>(m, S.ntile, w, S.rec.p, S.cnt.p, state), SVXG_COUNT_LAUNCH());
  if (v) (k_norm_rescale<<<nblk(m), kT, 0, st>>>(m, w, v, state), SVXG_COUNT_LAUNCH());
  return SVXG_OK;
}

// ---- strength (amg.cpp:324-330) ------------------------------------------------------------------
__global__ void k_fro_blocks(int64_t nnzb, const double* val, double* fro) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < nnzb) fro[k] = fro6(val + 36 * k);
}

__global__ void k_block_rows(int32_t n, const int32_t* rowptr, int32_t* brow) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) brow[k] = i;
}

// strong[k] for the round's theta: j != i && fro(A_ij) >= theta sqrt(dn_i dn_j)
__global__ void k_strong(int64_t nnzb, const int32_t* brow, const int32_t* col, const double* fro, const int32_t* rowptr,
                         double theta, uint8_t* strong) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= nnzb) return;
  const int32_t i = brow[k], j = col[k];
  const double dni = fro[rowptr[i]], dnj = fro[rowptr[j]];
  strong[k] = (j != i && fro[k] >= theta * sqrt(dni * dnj)) ? 1 : 0;
}

// ---- pass 1: the lexicographically first independent set, in rounds ---------------------------
// state: 0 undecided, 1 root, 2 non-root (isolated rows start as non-roots: amg.cpp:340)
__global__ void k_mis_init(int32_t n, const int32_t* rowptr, uint8_t* state, uint8_t* covered, int32_t* claim,
                           int32_t* claim2) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  state[i] = (rowptr[i + 1] - rowptr[i] <= 1) ? 2 : 0;
  covered[i] = 0;
  claim[i] = INT_MAX;
  claim2[i] = INT_MAX;
}

__global__ void k_mis_claim(int32_t n, const int32_t* rowptr, const int32_t* col, const uint8_t* strong,
                            const uint8_t* state, int32_t* claim) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || state[i] != 0) return;
  atomicMin(&claim[i], i);
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (strong[k]) atomicMin(&claim[col[k]], i);
}

__global__ void k_mis_decide(int32_t n, const int32_t* rowptr, const int32_t* col, const uint8_t* strong,
                             uint8_t* state, const uint8_t* covered, const int32_t* claim, int32_t* undecided) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || state[i] != 0) return;
  bool cov = covered[i] != 0;
  bool mine = claim[i] == i;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (strong[k]) {
      const int32_t x = col[k];
      cov = cov || covered[x] != 0;
      mine = mine && claim[x] == i;
    }
  if (cov) {
    state[i] = 2;
  } else if (mine) {
    state[i] = 3;  // (a root of this round: covers in k_mis_cover_claim)
  } else {
    atomicAdd(undecided, 1);
  }
}

// The cover of round r and the claims of round r + 1 in one launch, the claims double-buffered:
// round r's (claim_done) are reset while round r + 1's go to claim_next (reset by the previous
// such launch). A node decided in round r keeps a nonzero state, so only the still undecided
// claim.
__global__ void k_mis_cover_claim(int32_t n, const int32_t* rowptr, const int32_t* col, const uint8_t* strong,
                                  uint8_t* state, uint8_t* covered, int32_t* claim_done, int32_t* claim_next) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  claim_done[i] = INT_MAX;
  const uint8_t si = state[i];
  if (si == 3) {
    state[i] = 1;
    covered[i] = 1;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (strong[k]) covered[col[k]] = 1;
    return;
  }
  if (si != 0) return;
  atomicMin(&claim_next[i], i);
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (strong[k]) atomicMin(&claim_next[col[k]], i);
}

// All the rounds of a smaller level in one block (claim, decide, cover as above, a block barrier
// between them; the rounds end when a decide leaves no node undecided), instead of three launches
// a round and a host read every few rounds.
constexpr int32_t kMisSmall = 8192;
__global__ void __launch_bounds__(1024) k_mis_small(int32_t n, const int32_t* rowptr, const int32_t* col,
                                                    const uint8_t* strong, uint8_t* state, uint8_t* covered,
                                                    int32_t* claim) {
  for (int32_t round = 0; round <= n; ++round) {
    for (int32_t i = threadIdx.x; i < n; i += blockDim.x) {
      if (state[i] != 0) continue;
      atomicMin(&claim[i], i);
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) atomicMin(&claim[col[k]], i);
    }
    __syncthreads();
    int und = 0;
    for (int32_t i = threadIdx.x; i < n; i += blockDim.x) {
      if (state[i] != 0) continue;
      bool cov = covered[i] != 0;
      bool mine = claim[i] == i;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) {
          const int32_t x = col[k];
          cov = cov || covered[x] != 0;
          mine = mine && claim[x] == i;
        }
      if (cov) state[i] = 2;
      else if (mine) state[i] = 3;
      else und = 1;
    }
    const int any = __syncthreads_or(und);
    for (int32_t i = threadIdx.x; i < n; i += blockDim.x) {
      claim[i] = INT_MAX;
      if (state[i] != 3) continue;
      state[i] = 1;
      covered[i] = 1;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) covered[col[k]] = 1;
    }
    __syncthreads();
    if (!any) break;
  }
}

// The remaining rounds of a long level once few nodes are undecided, in one block over the list
// of those nodes (the same claim, decide and cover; decided nodes take no part in a round, so
// the rounds are the full-width ones). Claims are reset on every entry a round wrote.
__global__ void __launch_bounds__(1024) k_mis_tail(const int32_t* list, int32_t m, const int32_t* rowptr,
                                                   const int32_t* col, const uint8_t* strong, uint8_t* state,
                                                   uint8_t* covered, int32_t* claim) {
  for (int32_t round = 0; round <= m; ++round) {
    for (int32_t t = threadIdx.x; t < m; t += blockDim.x) {
      const int32_t i = list[t];
      if (state[i] != 0) continue;
      atomicMin(&claim[i], i);
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) atomicMin(&claim[col[k]], i);
    }
    __syncthreads();
    int und = 0;
    for (int32_t t = threadIdx.x; t < m; t += blockDim.x) {
      const int32_t i = list[t];
      if (state[i] != 0) continue;
      bool cov = covered[i] != 0;
      bool mine = claim[i] == i;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) {
          const int32_t x = col[k];
          cov = cov || covered[x] != 0;
          mine = mine && claim[x] == i;
        }
      if (cov) state[i] = 2;
      else if (mine) state[i] = 3;
      else und = 1;
    }
    const int any = __syncthreads_or(und);
    for (int32_t t = threadIdx.x; t < m; t += blockDim.x) {
      const int32_t i = list[t];
      claim[i] = INT_MAX;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) claim[col[k]] = INT_MAX;
    }
    __syncthreads();
    for (int32_t t = threadIdx.x; t < m; t += blockDim.x) {
      const int32_t i = list[t];
      if (state[i] != 3) continue;
      state[i] = 1;
      covered[i] = 1;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
        if (strong[k]) covered[col[k]] = 1;
    }
    __syncthreads();
    if (!any) break;
  }
}

// (a round of one block over the list costs about what three grid-wide launches cost once the
// list is this short)
constexpr int32_t kMisTail = 1024;

__global__ void k_undecided_flags(int32_t n, const uint8_t* state, int32_t* flag) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = state[i] == 0 ? 1 : 0;
}

__global__ void k_list_flagged(int32_t n, const int32_t* flag, const int32_t* pos, int32_t* out) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) out[pos[i]] = i;
}

__global__ void k_root_flags(int32_t n, const uint8_t* state, int32_t* flag) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = state[i] == 1 ? 1 : 0;
}

// agg1: roots' ranks on their N[r] (pass 1's result)
__global__ void k_agg_pass1(int32_t n, const int32_t* rowptr, const int32_t* col, const uint8_t* strong,
                            const uint8_t* state, const int32_t* rank, int32_t* agg1) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || state[i] != 1) return;
  const int32_t a = rank[i];
  agg1[i] = a;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (strong[k]) agg1[col[k]] = a;
}

// pass 2 (amg.cpp:351-366): the most strongly coupled aggregated neighbour (first in row order on ties)
__global__ void k_agg_pass2(int32_t n, const int32_t* rowptr, const int32_t* col, const double* fro,
                            const int32_t* agg1, int32_t* agg) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (agg1[i] >= 0) {
    agg[i] = agg1[i];
    return;
  }
  double best = -1.0;
  int32_t ba = -1;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int32_t j = col[k];
    if (j == i || agg1[j] < 0) continue;
    const double s = fro[k];
    if (s > best) {
      best = s;
      ba = agg1[j];
    }
  }
  agg[i] = ba;
}

// pass 3 (amg.cpp:367-384) flags: leftovers, isolated leftovers
__global__ void k_pass3_flags(int32_t n, const int32_t* rowptr, const int32_t* agg, int32_t* iso, int32_t* noniso) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool left = agg[i] < 0;
  const bool isolated = rowptr[i + 1] - rowptr[i] <= 1;
  iso[i] = (left && isolated) ? 1 : 0;
  noniso[i] = (left && !isolated) ? 1 : 0;
}

// an id is opened by every non-isolated leftover and by every eighth isolated one (group == 0, a
// batch of graphs: by every isolated one - eight of them may belong to eight graphs, and the
// batch's multigrid must not couple its graphs)
__global__ void k_pass3_alloc(int32_t n, const int32_t* iso, const int32_t* isorank, const int32_t* noniso,
                              int32_t group, int32_t* alloc, int32_t* group_first) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool opens = noniso[i] || (iso[i] && (!group || isorank[i] % 8 == 0));
  alloc[i] = opens ? 1 : 0;
  if (group && iso[i] && isorank[i] % 8 == 0) group_first[isorank[i] / 8] = i;
}

__global__ void k_pass3_assign(int32_t n, int32_t base, const int32_t* iso, const int32_t* isorank,
                               const int32_t* noniso, int32_t group, const int32_t* allocscan,
                               const int32_t* group_first, int32_t* agg) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (noniso[i] || (iso[i] && !group)) agg[i] = base + allocscan[i];
  else if (iso[i]) agg[i] = base + allocscan[group_first[isorank[i] / 8]];
}

// ---- coarse positions (amg.cpp:391-401) ------------------------------------------------------------
__global__ void k_count_members(int32_t n, const int32_t* agg, int32_t* cnt) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[agg[i]], 1);
}

__global__ void k_fill_members(int32_t n, const int32_t* agg, const int32_t* off, int32_t* cursor, int32_t* members) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t a = agg[i];
  members[off[a] + atomicAdd(&cursor[a], 1)] = i;
}

// per aggregate: members sorted, positions summed in node order, then times 1 / count
__global__ void k_coarse_pos(int32_t na, const int32_t* off, int32_t* members, const double* fpos, double* cpos) {
  const int32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= na) return;
  const int32_t e0 = off[a], e1 = off[a + 1];
  for (int32_t u = e0 + 1; u < e1; ++u) {
    const int32_t v = members[u];
    int32_t c = u - 1;
    while (c >= e0 && members[c] > v) {
      members[c + 1] = members[c];
      --c;
    }
    members[c + 1] = v;
  }
  double x = 0.0, y = 0.0, z = 0.0;
  for (int32_t u = e0; u < e1; ++u) {
    const int32_t i = members[u];
    x += fpos[3 * int64_t(i)];
    y += fpos[3 * int64_t(i) + 1];
    z += fpos[3 * int64_t(i) + 2];
  }
  const double s = 1.0 / (e1 - e0);
  cpos[3 * int64_t(a)] = x * s;
  cpos[3 * int64_t(a) + 1] = y * s;
  cpos[3 * int64_t(a) + 2] = z * s;
}

__global__ void k_offsets(int32_t n, const int32_t* agg, const double* fpos, const double* cpos, double* off3) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t a = agg[i];
  for (int c = 0; c < 3; ++c) off3[3 * int64_t(i) + c] = fpos[3 * int64_t(i) + c] - cpos[3 * int64_t(a) + c];
}

// ---- prolongation (amg.cpp:405-452) ----------------------------------------------------------------
// distinct coarse columns of fine row i: agg[i] and agg[col k] (all k when smoothed)
__device__ int32_t sorted_distinct(int32_t first, const int32_t* rowptr, const int32_t* col, const int32_t* agg,
                                   int32_t i, bool all, int32_t* out, int32_t cap) {
  int32_t m = 0;
  auto insert = [&](int32_t c) {
    int32_t p = 0;
    while (p < m && out[p] < c) ++p;
    if (p < m && out[p] == c) return;
    if (m >= cap) return;
    for (int32_t q = m; q > p; --q) out[q] = out[q - 1];
    out[p] = c;
    ++m;
  };
  insert(first);
  if (all)
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) insert(agg[col[k]]);
  return m;
}

__global__ void k_p_count(int32_t n, const int32_t* rowptr, const int32_t* col, const int32_t* agg, int smoothed,
                          int32_t* plen, int32_t* scratch, int32_t cap) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  plen[i] = sorted_distinct(agg[i], rowptr, col, agg, i, smoothed != 0, scratch + int64_t(rowptr[i]) + i, cap);
}

// 0.0 + x without an FP64 operation: x, with -0.0 made +0.0 (the reference's sums start at +0.0;
// the first addition changes nothing else for a finite or infinite x), by an integer test on the
// bits - the FP64 pipe bounds the products below
__device__ __forceinline__ double plus_zero(double x) {
  const long long b = __double_as_longlong(x);
  return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}

// rigid_block(r)[q][c] (blk6.cuh) with r = off3 row j, the same values without the array
__device__ __forceinline__ double rigid_entry(const double* off3, int32_t j, int q, int c) {
  if (q == c) return 1.0;
  const double* r = off3 + 3 * int64_t(j);
  switch (q * 6 + c) {
    case 4: return r[2];
    case 5: return -r[1];
    case 9: return -r[2];
    case 11: return r[0];
    case 15: return r[1];
    case 16: return -r[0];
    default: return 0.0;
  }
}

// (A rigid_block(r))[row][c]: mul6's sum over q with the rigid block's zero terms left out and
// its unit terms as plain additions. A zero product added to a sum that starts at +0.0 leaves it
// unchanged (the sum is never -0.0) when A is finite, and x * 1.0 is x: the same bits as the
// full sum for finite K, with 4 of its 12 FP64 operations at most.
__device__ __forceinline__ double a_rigid_entry(const double* A, int row, int c, const double* r) {
  const double* a = A + 6 * row;
  switch (c) {
    case 0:
    case 1:
    case 2: return plus_zero(a[c]);
    case 3: return (plus_zero(a[1] * -r[2]) + a[2] * r[1]) + a[3];
    case 4: return (plus_zero(a[0] * r[2]) + a[2] * -r[0]) + a[4];
    default: return (plus_zero(a[0] * -r[1]) + a[1] * r[0]) + a[5];
  }
}

// The smoothed prolongation rows (amg.cpp:405-452), a warp per fine row i, its P blocks in
// shared memory when it has at most kPSlots of them. The row's own aggregate block gets
// rigid_block(off_i); then, for the row's neighbours k in chunks of kPNb, T_k = A_ik rigid_block
// (off_j) and U_k = D_i^-1 T_k with the (k, entry) items spread over the lanes (GB300 issues FP64
// instructions for whole warps), and the block of aggregate agg[j] adds -omega U_k, neighbour by
// neighbour. Every entry gets the reference's sums (mul6's 6-term sums, the axpy) in its order;
// T's sums skip the rigid block's zero terms (a_rigid_entry).
constexpr int kPNb = 8;
constexpr int kPSlots = 16;
constexpr int kPWarps = 4;
__global__ void __launch_bounds__(32 * kPWarps) k_p_values(int32_t n, const int32_t* rowptr, const int32_t* col,
                                                           const double* val, const int32_t* agg, const double* off3,
                                                           const double* dinv, double omega, const int32_t* prow,
                                                           const int32_t* scratch, int32_t* pcol, double* pval) {
  __shared__ double t_sh[kPWarps][kPNb * 36], u_sh[kPWarps][kPNb * 36];
  __shared__ double acc_sh[kPWarps][kPSlots * 36];
  __shared__ int32_t slot_sh[kPWarps][kPNb];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t i = int32_t(blockIdx.x) * kPWarps + wid;
  if (i >= n) return;
  const int32_t e0 = prow[i], len = prow[i + 1] - e0;
  const int32_t* cols = scratch + int64_t(rowptr[i]) + i;
  for (int32_t e = lane; e < len; e += 32) pcol[e0 + e] = cols[e];
  const bool local = len <= kPSlots;
  double* acc = local ? acc_sh[wid] : pval + 36 * int64_t(e0);
  for (int32_t q = lane; q < 36 * len; q += 32) acc[q] = 0.0;
  const auto find = [&](int32_t c) {
    int32_t lo = 0, hi = len - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi) >> 1;
      if (cols[mid] < c) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  __syncwarp();
  {
    double* b = acc + 36 * int64_t(find(agg[i]));
    for (int q = lane; q < 36; q += 32) b[q] = b[q] + 1.0 * rigid_entry(off3, i, q / 6, q % 6);
  }
  __syncwarp();
  if (omega != 0.0) {
    const double* Di = dinv + 36 * int64_t(i);
    for (int32_t kb = rowptr[i]; kb < rowptr[i + 1]; kb += kPNb) {
      const int32_t nk = rowptr[i + 1] - kb < kPNb ? rowptr[i + 1] - kb : kPNb;
      if (lane < nk) slot_sh[wid][lane] = find(agg[col[kb + lane]]);
      for (int32_t it = lane; it < 36 * nk; it += 32) {
        const int32_t kl = it / 36, ent = it - 36 * kl;
        const int r = ent / 6, c = ent - 6 * r;
        t_sh[wid][it] = a_rigid_entry(val + 36 * int64_t(kb + kl), r, c, off3 + 3 * int64_t(col[kb + kl]));
      }
      __syncwarp();
      for (int32_t it = lane; it < 36 * nk; it += 32) {
        const int32_t kl = it / 36, ent = it - 36 * kl;
        const int r = ent / 6, c = ent - 6 * r;
        const double* T = t_sh[wid] + 36 * kl;
        double s = plus_zero(Di[r * 6] * T[c]);
        for (int q = 1; q < 6; ++q) s += Di[r * 6 + q] * T[q * 6 + c];
        u_sh[wid][it] = s;
      }
      __syncwarp();
      for (int32_t kl = 0; kl < nk; ++kl) {
        double* b = acc + 36 * int64_t(slot_sh[wid][kl]);
        for (int q = lane; q < 36; q += 32) b[q] = b[q] + -omega * u_sh[wid][36 * kl + q];
        __syncwarp();
      }
    }
  }
  if (local)
    for (int32_t q = lane; q < 36 * len; q += 32) pval[36 * int64_t(e0) + q] = acc[q];
}

// build work of the products: 6 |P row col(k)| for every block k of A
__global__ void k_work_ap(int64_t nnzb, const int32_t* col, const int32_t* prow, unsigned long long* acc) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned long long w = 0;
  if (k < nnzb) {
    const int32_t j = col[k];
    w = 6ull * unsigned(prow[j + 1] - prow[j]);
  }
  for (int d = 16; d > 0; d >>= 1) w += __shfl_xor_sync(0xffffffffu, w, d);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(acc, w);
}

// ---- restriction lists (amg.cpp:461-470) ---------------------------------------------------------
__global__ void k_r_count(int64_t pnnz, const int32_t* pcol, int32_t* cnt) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < pnnz) atomicAdd(&cnt[pcol[e]], 1);
}

__global__ void k_r_fill(int32_t n, const int32_t* prow, const int32_t* pcol, const int32_t* rrow, int32_t* cursor,
                         int32_t* rent_e) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int32_t e = prow[i]; e < prow[i + 1]; ++e) {
    const int32_t c = pcol[e];
    rent_e[rrow[c] + atomicAdd(&cursor[c], 1)] = e;
  }
}

// per coarse row: entries by P index (= by fine row, then P index), and their fine rows
__global__ void k_r_sort(int32_t na, const int32_t* rrow, int32_t* rent_e, int32_t* rent_i, const int32_t* erow) {
  const int32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= na) return;
  const int32_t e0 = rrow[a], e1 = rrow[a + 1];
  for (int32_t u = e0 + 1; u < e1; ++u) {
    const int32_t v = rent_e[u];
    int32_t c = u - 1;
    while (c >= e0 && rent_e[c] > v) {
      rent_e[c + 1] = rent_e[c];
      --c;
    }
    rent_e[c + 1] = v;
  }
  for (int32_t u = e0; u < e1; ++u) rent_i[u] = erow[rent_e[u]];
}

__global__ void k_entry_rows(int32_t n, const int32_t* prow, int32_t* erow) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int32_t e = prow[i]; e < prow[i + 1]; ++e) erow[e] = i;
}

// ---- Galerkin product (amg.cpp:472-529) ------------------------------------------------------------
// A P by fine row: distinct coarse columns over (k, e), sorted
__global__ void k_ap_count(int32_t n, const int32_t* rowptr, const int32_t* col, const int32_t* prow,
                           const int32_t* pcol, int32_t* aplen, int32_t* scratch, const int64_t* soff, int32_t cap) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t* out = scratch + soff[i];
  int32_t m = 0;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int32_t j = col[k];
    for (int32_t e = prow[j]; e < prow[j + 1]; ++e) {
      const int32_t c = pcol[e];
      int32_t p = 0;
      while (p < m && out[p] < c) ++p;
      if (p < m && out[p] == c) continue;
      if (m >= cap) continue;
      for (int32_t q = m; q > p; --q) out[q] = out[q - 1];
      out[p] = c;
      ++m;
    }
  }
  aplen[i] = m;
}

// (one warp per row: lane l owns entries l and, for l < 4, 32 + l of every 6x6 product; each
// entry is summed over q in order and added to its block as mul6_add does - the same additions)
__device__ __forceinline__ void warp_mul6_add(bool trans, const double* __restrict__ A, const double* __restrict__ B,
                                              double* C, int lane) {
  for (int ent = lane; ent < 36; ent += 32) {
    const int r = ent / 6, c = ent - 6 * (ent / 6);
    double s = 0.0;
    for (int q = 0; q < 6; ++q) s += (trans ? A[q * 6 + r] : A[r * 6 + q]) * B[q * 6 + c];
    C[ent] = C[ent] + s;
  }
}

// The same A P rows, accumulated in shared memory when a row has at most kAccSlots blocks (the
// row's blocks are read-modify-written once per product; in shared memory that round trip is
// short). For each block A_ik of the row, the products with the blocks of P's row k are spread
// over the lanes as (P entry, output entry) items: GB300 issues FP64 instructions for whole warps,
// so the lanes are kept busy rather than one lane per output entry (36 entries: a pass of 32 and
// a pass of 4). Every output entry receives the same sums in the same order as warp_mul6_add:
// the k's in row order, each entry one 6-term sum. Longer rows go through global memory.
constexpr int kAccSlots = 40;
constexpr int kAccWarps = 4;
__global__ void __launch_bounds__(32 * kAccWarps) k_ap_values_acc(int32_t n, const int32_t* rowptr, const int32_t* col,
                                                                  const double* val, const int32_t* prow,
                                                                  const int32_t* pcol, const double* pval,
                                                                  const int32_t* aprow, const int32_t* scratch,
                                                                  const int64_t* soff, int32_t* apcol, double* apval) {
  __shared__ double acc_sh[kAccWarps][kAccSlots * 36];
  __shared__ int32_t col_sh[kAccWarps][kAccSlots];
  __shared__ int32_t slot_sh[kAccWarps][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t i = int32_t(blockIdx.x) * kAccWarps + wid;
  if (i >= n) return;
  const int32_t e0 = aprow[i], e1 = aprow[i + 1], len = e1 - e0;
  const bool local = len <= kAccSlots;
  double* acc = local ? acc_sh[wid] : apval + 36 * int64_t(e0);
  const int32_t* cols = local ? col_sh[wid] : apcol + e0;
  for (int32_t e = lane; e < len; e += 32) {
    const int32_t c = scratch[soff[i] + e];
    apcol[e0 + e] = c;
    if (local) col_sh[wid][e] = c;
  }
  for (int32_t q = lane; q < 36 * len; q += 32) acc[q] = 0.0;
  __syncwarp();
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int32_t j = col[k];
    const double* A = val + 36 * int64_t(k);
    for (int32_t pb = prow[j]; pb < prow[j + 1]; pb += 32) {
      const int32_t np = prow[j + 1] - pb < 32 ? prow[j + 1] - pb : 32;
      if (lane < np) {
        const int32_t cc = pcol[pb + lane];
        int32_t lo = 0, hi = len - 1;
        while (lo < hi) {
          const int32_t mid = (lo + hi) >> 1;
          if (cols[mid] < cc) lo = mid + 1;
          else hi = mid;
        }
        slot_sh[wid][lane] = lo;
      }
      __syncwarp();
      for (int32_t it = lane; it < 36 * np; it += 32) {
        const int32_t el = it / 36, ent = it - 36 * el;
        const int r = ent / 6, c = ent - 6 * r;
        const double* B = pval + 36 * int64_t(pb + el);
        double s0 = plus_zero(A[r * 6] * B[c]);
        for (int q = 1; q < 6; ++q) s0 += A[r * 6 + q] * B[q * 6 + c];
        double* C = acc + 36 * int64_t(slot_sh[wid][el]) + ent;
        *C = *C + s0;
      }
      __syncwarp();
    }
  }
  if (local)
    for (int32_t q = lane; q < 36 * len; q += 32) apval[36 * int64_t(e0) + q] = acc[q];
}

// A P a warp per block of A P for levels of few rows (too few warps to fill the GPU a row each):
// block k = (i, J) has its 36 entries in the lanes' registers; the warp walks A's row i in order
// and, for each block A_ij, finds J in P's row j (32 entries a step, by ballot; a row holds a
// column at most once) and adds the entry's 6-term sum - every entry receives one 6-term sum per
// A block whose P row holds J, in row order: k_ap_values_acc's sums.
constexpr int kApWarps = 4;
__global__ void __launch_bounds__(32 * kApWarps) k_ap_values_warp(int32_t n, int64_t apnnz, const int32_t* rowptr,
                                                                  const int32_t* col, const double* val,
                                                                  const int32_t* prow, const int32_t* pcol,
                                                                  const double* pval, const int32_t* aprow,
                                                                  const int32_t* scratch, const int64_t* soff,
                                                                  int32_t* apcol, double* apval) {
  const int lane = threadIdx.x & 31;
  const int64_t k = int64_t(blockIdx.x) * kApWarps + (threadIdx.x >> 5);
  if (k >= apnnz) return;
  // (the row of block k: the last i with aprow[i] <= k)
  int32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (aprow[mid] <= k) lo = mid;
    else hi = mid - 1;
  }
  const int32_t i = lo;
  const int32_t J = scratch[soff[i] + (k - aprow[i])];
  if (lane == 0) apcol[k] = J;
  const int ra = lane / 6, ca = lane - 6 * (lane / 6);
  const bool two = lane < 4;
  const int rb = (lane + 32) / 6, cb = (lane + 32) - 6 * ((lane + 32) / 6);
  double a0 = 0.0, a1 = 0.0;
  for (int32_t kk = rowptr[i]; kk < rowptr[i + 1]; ++kk) {
    const int32_t j = col[kk];
    const int32_t p0 = prow[j], np = prow[j + 1] - p0;
    int32_t found = -1;
    for (int32_t b = 0; b < np; b += 32) {
      const bool hit = b + lane < np && pcol[p0 + b + lane] == J;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (m) {
        found = p0 + b + __ffs(int(m)) - 1;
        break;
      }
    }
    if (found < 0) continue;
    const double* A = val + 36 * int64_t(kk);
    const double* B = pval + 36 * int64_t(found);
    double s0 = plus_zero(A[ra * 6] * B[ca]);
    for (int q = 1; q < 6; ++q) s0 += A[ra * 6 + q] * B[q * 6 + ca];
    a0 = a0 + s0;
    if (two) {
      double s1 = plus_zero(A[rb * 6] * B[cb]);
      for (int q = 1; q < 6; ++q) s1 += A[rb * 6 + q] * B[q * 6 + cb];
      a1 = a1 + s1;
    }
  }
  apval[36 * k + lane] = a0;
  if (two) apval[36 * k + 32 + lane] = a1;
}

// The coarse rows C = P^T (A P) in the same way: a warp per coarse row, accumulated in shared
// memory when it has at most kAccSlots blocks. For each restriction entry (fine row i, block P_iI)
// the blocks of A P's row i are taken 32 at a time and their (block, C entry) items spread over
// the lanes; each C entry receives one 6-term sum per restriction entry, in restriction order.
__global__ void __launch_bounds__(32 * kAccWarps) k_c_values_acc(int32_t na, const int32_t* rrow, const int32_t* rent_i,
                                                                 const int32_t* rent_e, const double* pval,
                                                                 const int32_t* aprow, const int32_t* apcol,
                                                                 const double* apval, const int32_t* crow,
                                                                 const int32_t* scratch, const int64_t* soff,
                                                                 int32_t* ccol, double* cval, double scale) {
  __shared__ double acc_sh[kAccWarps][kAccSlots * 36];
  __shared__ int32_t col_sh[kAccWarps][kAccSlots];
  __shared__ int32_t slot_sh[kAccWarps][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t I = int32_t(blockIdx.x) * kAccWarps + wid;
  if (I >= na) return;
  const int32_t c0 = crow[I], c1 = crow[I + 1], len = c1 - c0;
  const bool local = len <= kAccSlots;
  double* acc = local ? acc_sh[wid] : cval + 36 * int64_t(c0);
  const int32_t* cols = local ? col_sh[wid] : ccol + c0;
  for (int32_t c = lane; c < len; c += 32) {
    const int32_t v = scratch[soff[I] + c];
    ccol[c0 + c] = v;
    if (local) col_sh[wid][c] = v;
  }
  for (int32_t q = lane; q < 36 * len; q += 32) acc[q] = 0.0;
  __syncwarp();
  for (int32_t r = rrow[I]; r < rrow[I + 1]; ++r) {
    const int32_t i = rent_i[r];
    const double* Pi = pval + 36 * int64_t(rent_e[r]);
    for (int32_t eb = aprow[i]; eb < aprow[i + 1]; eb += 32) {
      const int32_t ne = aprow[i + 1] - eb < 32 ? aprow[i + 1] - eb : 32;
      if (lane < ne) {
        const int32_t J = apcol[eb + lane];
        int32_t slot;
        if (J == I) {
          slot = 0;
        } else {
          int32_t lo = 1, hi = len - 1;
          while (lo < hi) {
            const int32_t mid = (lo + hi) >> 1;
            if (cols[mid] < J) lo = mid + 1;
            else hi = mid;
          }
          slot = lo;
        }
        slot_sh[wid][lane] = slot;
      }
      __syncwarp();
      for (int32_t it = lane; it < 36 * ne; it += 32) {
        const int32_t el = it / 36, ent = it - 36 * el;
        const int rr = ent / 6, cc = ent - 6 * rr;
        const double* B = apval + 36 * int64_t(eb + el);
        double sacc = plus_zero(Pi[rr] * B[cc]);
        for (int q = 1; q < 6; ++q) sacc += Pi[q * 6 + rr] * B[q * 6 + cc];
        double* C = acc + 36 * int64_t(slot_sh[wid][el]) + ent;
        *C = *C + sacc;
      }
      __syncwarp();
    }
  }
  if (scale != 1.0)
    for (int32_t q = lane; q < 36 * len; q += 32) acc[q] *= scale;
  __syncwarp();
  if (local)
    for (int32_t q = lane; q < 36 * len; q += 32) cval[36 * int64_t(c0) + q] = acc[q];
}

constexpr int32_t kFewRows = 2432;  // (coarse rows: 16 warps on each of 152 SMs)
constexpr int32_t kFewRowsAP = 2432;  // (fine rows of A P likewise)

// C = P^T (A P) a warp per block of C: block k = (I, J) - I its coarse row, J its column - has
// its 36 entries in the lanes' registers (entry lane, and 32 + lane for the first four lanes).
// The warp walks row I's restriction entries (fine row i, block P_iI) in restriction order, finds
// J in A P's row i (32 columns a step, by ballot; a row holds a column at most once) and adds
// the entry's 6-term sum P_iI^T (A P)_iJ: every C entry receives one 6-term sum per restriction
// entry whose A P row holds J, in restriction order - the sums of the row-at-a-time forms, with
// no barrier, no shared accumulator and a warp for each block of C (coarse levels of a few
// hundred rows still give thousands of warps).
constexpr int kCWarps = 4;
__global__ void __launch_bounds__(32 * kCWarps) k_c_values_warp(int32_t na, int64_t cnnz, const int32_t* rrow,
                                                                const int32_t* rent_i, const int32_t* rent_e,
                                                                const double* pval, const int32_t* aprow,
                                                                const int32_t* apcol, const double* apval,
                                                                const int32_t* crow, const int32_t* scratch,
                                                                const int64_t* soff, int32_t* ccol, double* cval,
                                                                double scale) {
  const int lane = threadIdx.x & 31;
  const int64_t k = int64_t(blockIdx.x) * kCWarps + (threadIdx.x >> 5);
  if (k >= cnnz) return;
  // (the coarse row of block k: the last I with crow[I] <= k)
  int32_t lo = 0, hi = na - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (crow[mid] <= k) lo = mid;
    else hi = mid - 1;
  }
  const int32_t I = lo;
  const int32_t J = scratch[soff[I] + (k - crow[I])];
  if (lane == 0) ccol[k] = J;
  const int ra = lane / 6, ca = lane - 6 * (lane / 6);
  const bool two = lane < 4;
  const int rb = (lane + 32) / 6, cb = (lane + 32) - 6 * ((lane + 32) / 6);
  double a0 = 0.0, a1 = 0.0;
  for (int32_t r = rrow[I]; r < rrow[I + 1]; ++r) {
    const int32_t i = rent_i[r];
    const int32_t e0 = aprow[i], ne = aprow[i + 1] - e0;
    int32_t found = -1;
    for (int32_t b = 0; b < ne; b += 32) {
      const bool hit = b + lane < ne && apcol[e0 + b + lane] == J;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (m) {
        found = e0 + b + __ffs(int(m)) - 1;
        break;
      }
    }
    if (found < 0) continue;
    const double* Pi = pval + 36 * int64_t(rent_e[r]);
    const double* B = apval + 36 * int64_t(found);
    double s0 = plus_zero(Pi[ra] * B[ca]);
    for (int q = 1; q < 6; ++q) s0 += Pi[q * 6 + ra] * B[q * 6 + ca];
    a0 = a0 + s0;
    if (two) {
      double s1 = plus_zero(Pi[rb] * B[cb]);
      for (int q = 1; q < 6; ++q) s1 += Pi[q * 6 + rb] * B[q * 6 + cb];
      a1 = a1 + s1;
    }
  }
  if (scale != 1.0) {
    a0 *= scale;
    a1 *= scale;
  }
  cval[36 * k + lane] = a0;
  if (two) cval[36 * k + 32 + lane] = a1;
}

// build work of P^T (A P): 6 |P row i| |AP row i|
__global__ void k_work_rap(int32_t n, const int32_t* prow, const int32_t* aprow, unsigned long long* acc) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long w = 0;
  if (i < n) w = 6ull * unsigned(prow[i + 1] - prow[i]) * unsigned(aprow[i + 1] - aprow[i]);
  for (int d = 16; d > 0; d >>= 1) w += __shfl_xor_sync(0xffffffffu, w, d);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(acc, w);
}

// coarse row I: distinct columns over its restriction entries' A P rows; diagonal first, then
// ascending (Bsr6Builder::finish)
__global__ void k_c_count(int32_t na, const int32_t* rrow, const int32_t* rent_i, const int32_t* aprow,
                          const int32_t* apcol, int32_t* clen, int32_t* scratch, const int64_t* soff, int32_t cap) {
  const int32_t I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= na) return;
  int32_t* out = scratch + soff[I];
  int32_t m = 0;
  for (int32_t r = rrow[I]; r < rrow[I + 1]; ++r) {
    const int32_t i = rent_i[r];
    for (int32_t e = aprow[i]; e < aprow[i + 1]; ++e) {
      const int32_t c = apcol[e];
      int32_t p = 0;
      while (p < m && out[p] < c) ++p;
      if (p < m && out[p] == c) continue;
      if (m >= cap) continue;
      for (int32_t q = m; q > p; --q) out[q] = out[q - 1];
      out[p] = c;
      ++m;
    }
  }
  // (the diagonal to the front)
  int32_t p = 0;
  while (p < m && out[p] != I) ++p;
  if (p < m) {
    for (int32_t q = p; q > 0; --q) out[q] = out[q - 1];
    out[0] = I;
    clen[I] = m;
  } else {
    for (int32_t q = m; q > 0; --q) out[q] = out[q - 1];
    out[0] = I;
    clen[I] = m + 1;
  }
}

// The same columns for coarse levels of at most kBitmapCols rows, one warp per coarse row: the
// row's candidate columns are marked in a bitmap in shared memory, which is then read in column
// order (the serial insertion above costs the candidates times the row length per thread, and
// coarse rows are long).
constexpr int32_t kBitmapCols = 8192;
constexpr int kBitmapWarps = 4;

// the set bits of bm[0, words) as ascending column indices into out (whole warp); returns the count
__device__ __forceinline__ int32_t warp_emit_bitmap(const unsigned* bm, int32_t words, int32_t* out, int lane) {
  int32_t base = 0;
  for (int32_t q0 = 0; q0 < words; q0 += 32) {
    const int32_t q = q0 + lane;
    const unsigned w = q < words ? bm[q] : 0u;
    const int cnt = __popc(w);
    int pre = cnt;
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, pre, d);
      if (lane >= d) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31);
    int32_t pos = base + pre - cnt;
    for (unsigned x = w; x; x &= x - 1) out[pos++] = 32 * q + (__ffs(x) - 1);
    base += total;
  }
  return base;
}
__global__ void __launch_bounds__(32 * kBitmapWarps) k_c_count_bitmap(int32_t na, const int32_t* rrow,
                                                                      const int32_t* rent_i, const int32_t* aprow,
                                                                      const int32_t* apcol, int32_t* clen,
                                                                      int32_t* scratch, const int64_t* soff) {
  __shared__ unsigned bits[kBitmapWarps][kBitmapCols / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t I = int32_t(blockIdx.x) * kBitmapWarps + wid;
  if (I >= na) return;  // (whole warps leave together)
  unsigned* bm = bits[wid];
  const int32_t words = (na + 31) / 32;
  for (int32_t q = lane; q < words; q += 32) bm[q] = 0u;
  __syncwarp();
  for (int32_t r = rrow[I]; r < rrow[I + 1]; ++r) {
    const int32_t i = rent_i[r];
    for (int32_t e = aprow[i] + lane; e < aprow[i + 1]; e += 32) {
      const int32_t c = apcol[e];
      atomicOr(&bm[c >> 5], 1u << (c & 31));
    }
  }
  __syncwarp();
  // the diagonal first, then the other columns ascending
  const bool has_diag = (bm[I >> 5] >> (I & 31)) & 1u;
  if (has_diag && lane == 0) bm[I >> 5] &= ~(1u << (I & 31));
  __syncwarp();
  int32_t* out = scratch + soff[I];
  if (lane == 0) out[0] = I;
  const int32_t len = 1 + warp_emit_bitmap(bm, words, out + 1, lane);
  if (lane == 0) clen[I] = len;
}

// A P's columns per fine row for levels of at most kBitmapCols coarse nodes (one warp per row)
__global__ void __launch_bounds__(32 * kBitmapWarps) k_ap_count_bitmap(int32_t n, int32_t na, const int32_t* rowptr,
                                                                       const int32_t* col, const int32_t* prow,
                                                                       const int32_t* pcol, int32_t* aplen,
                                                                       int32_t* scratch, const int64_t* soff) {
  __shared__ unsigned bits[kBitmapWarps][kBitmapCols / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t i = int32_t(blockIdx.x) * kBitmapWarps + wid;
  if (i >= n) return;
  unsigned* bm = bits[wid];
  const int32_t words = (na + 31) / 32;
  for (int32_t q = lane; q < words; q += 32) bm[q] = 0u;
  __syncwarp();
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int32_t j = col[k];
    for (int32_t e = prow[j] + lane; e < prow[j + 1]; e += 32) {
      const int32_t c = pcol[e];
      atomicOr(&bm[c >> 5], 1u << (c & 31));
    }
  }
  __syncwarp();
  const int32_t len = warp_emit_bitmap(bm, words, scratch + soff[i], lane);
  if (lane == 0) aplen[i] = len;
}

__global__ void k_c_values(int32_t na, const int32_t* rrow, const int32_t* rent_i, const int32_t* rent_e,
                           const double* pval, const int32_t* aprow, const int32_t* apcol, const double* apval,
                           const int32_t* crow, const int32_t* scratch, const int64_t* soff, int32_t* ccol,
                           double* cval, double scale) {
  const int lane = threadIdx.x & 31;
  const int32_t I = int32_t((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  if (I >= na) return;
  const int32_t c0 = crow[I], c1 = crow[I + 1];
  for (int32_t c = c0 + lane; c < c1; c += 32) ccol[c] = scratch[soff[I] + (c - c0)];
  for (int64_t q = 36 * int64_t(c0) + lane; q < 36 * int64_t(c1); q += 32) cval[q] = 0.0;
  __syncwarp();
  for (int32_t r = rrow[I]; r < rrow[I + 1]; ++r) {
    const int32_t i = rent_i[r];
    const double* Pi = pval + 36 * int64_t(rent_e[r]);
    for (int32_t e = aprow[i]; e < aprow[i + 1]; ++e) {
      const int32_t J = apcol[e];
      int32_t slot;
      if (J == I) {
        slot = c0;
      } else {
        int32_t lo = c0 + 1, hi = c1 - 1;
        while (lo < hi) {
          const int32_t mid = (lo + hi) >> 1;
          if (ccol[mid] < J) lo = mid + 1;
          else hi = mid;
        }
        slot = lo;
      }
      warp_mul6_add(true, Pi, apval + 36 * int64_t(e), cval + 36 * int64_t(slot), lane);
      __syncwarp();
    }
  }
  if (scale != 1.0)
    for (int64_t q = 36 * int64_t(c0) + lane; q < 36 * int64_t(c1); q += 32) cval[q] *= scale;
}

// per-row scratch offsets: sum over a row's products of the candidate counts (an upper bound)
__global__ void k_ap_bound(int32_t n, const int32_t* rowptr, const int32_t* col, const int32_t* prow, int32_t* bound) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t b = 0;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) b += prow[col[k] + 1] - prow[col[k]];
  bound[i] = b;
}

__global__ void k_c_bound(int32_t na, const int32_t* rrow, const int32_t* rent_i, const int32_t* aprow,
                          int32_t* bound) {
  const int32_t I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= na) return;
  int32_t b = 1;
  for (int32_t r = rrow[I]; r < rrow[I + 1]; ++r) b += aprow[rent_i[r] + 1] - aprow[rent_i[r]];
  bound[I] = b;
}

__global__ void k_widen_offsets(int32_t n, const int32_t* scan32, int64_t* off) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) off[i] = int64_t(scan32[i]);
}

// ---- the coarsest level's dense factor (amg.cpp:535-578) ---------------------------------------
// one thread per (row, entry of a 6x6 block): a row's columns are distinct, so each entry of C is
// written once over the zeroed matrix
__global__ void k_dense_fill(int32_t nc, const int32_t* rowptr, const int32_t* col, const double* val, int32_t m,
                             double* C) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= 36 * int64_t(nc)) return;
  const int32_t i = int32_t(t / 36);
  const int e = int(t % 36), r = e / 6, c = e % 6;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    C[int64_t(6 * i + r) * m + (6 * col[k] + c)] += val[36 * int64_t(k) + e];
}

// ---- host-side steps ---------------------------------------------------------------------------

int copy_to_host(Problem& P, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return SVXG_OK;
  SVXG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

// offsets of per-row scratch regions: an exclusive scan of the n bounds (bound[n] = 0)
int offsets64(Problem& P, const int32_t* bound, int32_t n, int64_t* off, int64_t* total) {
  int32_t* scan32 = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&scan32), sizeof(int32_t) * (size_t(n) + 1), P.stream));
  int32_t t = 0;
  int e = exclusive_scan_i32(P, bound, scan32, int64_t(n) + 1, &t);
  if (!e) (k_widen_offsets<<<nblk(int64_t(n) + 1), kT, 0, P.stream>>>(n, scan32, off), SVXG_COUNT_LAUNCH());
  cudaFreeAsync(scan32, P.stream);
  if (e) return e;
  if (t < 0) {
    set_error("multigrid setup: product scratch beyond 2^31 entries");
    return SVXG_ERR_NOMEM;
  }
  *total = t;
  return SVXG_OK;
}

int finalize_level(Problem& P, Level& L, bool* ok) {
  *ok = false;
  TRY(P.mem.alloc(&L.dinv, size_t(L.A.n) * 36));
  Tmp<int32_t> fail(P.stream);
  TRY(fail.alloc(1));
  SVXG_CUDA(cudaMemsetAsync(fail.p, 0, sizeof(int32_t), P.stream));
  if (L.A.n > 0) (k_dinv<<<nblk(L.A.n), kT, 0, P.stream>>>(L.A.n, L.A.rowptr, L.A.val, L.dinv, fail.p), SVXG_COUNT_LAUNCH());
  int32_t f = 0;
  TRY(copy_to_host(P, &f, fail.p, sizeof(int32_t)));
  P.amg_build_work += 12 * int64_t(L.A.n);
  *ok = f == 0;
  return SVXG_OK;
}

// estimate_lmax of a level (amg.cpp:256-275), the value the reference computes
int estimate_lmax(Problem& P, const Level& L, double* out) {
  const int32_t n = L.A.n;
  P.amg_build_work += 15 * (L.A.nnzb + n);
  const int64_t m = 6 * int64_t(n);
  Tmp<double> v(P.stream), w(P.stream), st(P.stream);
  NormScratch ns(P.stream);
  TRY(v.alloc(size_t(m)));
  TRY(w.alloc(size_t(m)));
  TRY(st.alloc(3));
  TRY(ns.alloc(m));
  const double init[3] = {1.0, 0.0, 0.0};
  SVXG_CUDA(cudaMemcpyAsync(st.p, init, sizeof(init), cudaMemcpyHostToDevice, P.stream));
  (k_lmax_init<<<nblk(m), kT, 0, P.stream>>>(m, v.p), SVXG_COUNT_LAUNCH());
  const unsigned ab = unsigned((m + 6 * kApplyNodes - 1) / (6 * kApplyNodes));
  if (m <= exact::kTile) {
    Tmp<unsigned> counter(P.stream);
    TRY(counter.alloc(1));
    SVXG_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned), P.stream));
    const unsigned sb = unsigned((n + exact::kThreads / 32 - 1) / (exact::kThreads / 32));
    for (int it = 0; it < 15; ++it)
      (k_lmax_step_small<<<sb, exact::kThreads, 0, P.stream>>>(n, L.A.rowptr, L.A.col, L.A.val, L.dinv, v.p, w.p,
                                                               ns.rec.p, ns.cnt.p, counter.p, st.p),
       SVXG_COUNT_LAUNCH());
  }
#ifdef SVXG_FAST_SETUP
  const unsigned fb = unsigned(std::min<int64_t>(kFastNormBlocks, (m + kFastNormT - 1) / kFastNormT));
  Tmp<double> part(P.stream);
  Tmp<unsigned> fcounter(P.stream);
  if (m > exact::kTile) {
    TRY(part.alloc(fb));
    TRY(fcounter.alloc(1));
    SVXG_CUDA(cudaMemsetAsync(fcounter.p, 0, sizeof(unsigned), P.stream));
  }
#endif
  for (int it = 0; m > exact::kTile && it < 15; ++it) {
    if (n <= kApplyRowsMax)
      (k_lmax_apply_rows<<<unsigned((n + kApplyWarps - 1) / kApplyWarps), 32 * kApplyWarps, 0, P.stream>>>(
           n, L.A.rowptr, L.A.col, L.A.val, L.dinv, v.p, w.p, st.p),
       SVXG_COUNT_LAUNCH());
    else
      (k_lmax_apply<<<ab, 6 * kApplyNodes, 0, P.stream>>>(n, L.A.rowptr, L.A.col, L.A.val, L.dinv, v.p, w.p, st.p),
       SVXG_COUNT_LAUNCH());
#ifdef SVXG_FAST_SETUP
    (k_norm_fast<<<fb, kFastNormT, 0, P.stream>>>(m, w.p, part.p, fcounter.p, st.p), SVXG_COUNT_LAUNCH());
    (k_norm_rescale<<<nblk(m), kT, 0, P.stream>>>(m, w.p, v.p, st.p), SVXG_COUNT_LAUNCH());
#else
    TRY(launch_norm(P.stream, m, w.p, v.p, st.p, ns));
#endif
  }
  SVXG_CUDA(cudaGetLastError());
  double h[3];
  TRY(copy_to_host(P, h, st.p, sizeof(h)));
  *out = 1.1 * h[0];
  return SVXG_OK;
}

// Amg::coarsen (amg.cpp:320-533): appends level l + 1; *made = false when coarsening stops
int coarsen(Problem& P, size_t l, bool smoothed, bool* made) {
  *made = false;
  cudaStream_t st = P.stream;
  const svxg_amg_options& opt = P.opt.amg;
  const int32_t n = P.lv[l].A.n;
  const int64_t nnzb = P.lv[l].A.nnzb;
  {
    const Bsr& A = P.lv[l].A;
    (void)A;
  }
  Tmp<double> fro(st);
  Tmp<int32_t> brow(st), agg1(st), flag(st), rank(st), claim(st), claim2(st), undecided(st);
  Tmp<uint8_t> strong(st), state(st), covered(st);
  TRY(fro.alloc(size_t(nnzb)));
  TRY(brow.alloc(size_t(nnzb)));
  TRY(strong.alloc(size_t(nnzb)));
  TRY(state.alloc(size_t(n)));
  TRY(covered.alloc(size_t(n)));
  TRY(claim.alloc(size_t(n)));
  TRY(claim2.alloc(size_t(n)));
  TRY(agg1.alloc(size_t(n)));
  TRY(flag.alloc(size_t(n) + 1));
  TRY(rank.alloc(size_t(n) + 1));
  TRY(undecided.alloc(8));
  Tmp<int32_t> iso(st), noniso(st), isorank(st), alloc(st), allocscan(st), gfirst(st);
  TRY(iso.alloc(size_t(n) + 1));
  TRY(noniso.alloc(size_t(n) + 1));
  TRY(isorank.alloc(size_t(n) + 1));
  TRY(alloc.alloc(size_t(n) + 1));
  TRY(allocscan.alloc(size_t(n) + 1));
  TRY(gfirst.alloc(size_t(n) / 8 + 2));
  int32_t* agg = nullptr;
  TRY(P.mem.alloc(&agg, size_t(n)));
  {
    const Bsr& A = P.lv[l].A;
    (k_fro_blocks<<<nblk(nnzb), kT, 0, st>>>(nnzb, A.val, fro.p), SVXG_COUNT_LAUNCH());
    (k_block_rows<<<nblk(n), kT, 0, st>>>(n, A.rowptr, brow.p), SVXG_COUNT_LAUNCH());
  }
  double theta = opt.strength;
  int32_t na = 0;
  for (int round = 0;; ++round) {
    const Bsr& A = P.lv[l].A;
    (k_strong<<<nblk(nnzb), kT, 0, st>>>(nnzb, brow.p, A.col, fro.p, A.rowptr, theta, strong.p), SVXG_COUNT_LAUNCH());
    (k_mis_init<<<nblk(n), kT, 0, st>>>(n, A.rowptr, state.p, covered.p, claim.p, claim2.p), SVXG_COUNT_LAUNCH());
    // rounds in batches of kBatch (a round after the last decision changes nothing), one host
    // read per batch: the last round's count of undecided nodes; two launches a round (decide,
    // then cover + the next round's claims)
    constexpr int kBatch = 8;
    int32_t* cur = claim.p;
    int32_t* nxt = claim2.p;
    if (n <= kMisSmall)
      (k_mis_small<<<1, 1024, 0, st>>>(n, A.rowptr, A.col, strong.p, state.p, covered.p, claim.p), SVXG_COUNT_LAUNCH());
    else
      (k_mis_claim<<<nblk(n), kT, 0, st>>>(n, A.rowptr, A.col, strong.p, state.p, cur), SVXG_COUNT_LAUNCH());
    for (int guard = 0; n > kMisSmall && guard <= n; guard += kBatch) {
      SVXG_CUDA(cudaMemsetAsync(undecided.p, 0, sizeof(int32_t) * kBatch, st));
      for (int b = 0; b < kBatch; ++b) {
        (k_mis_decide<<<nblk(n), kT, 0, st>>>(n, A.rowptr, A.col, strong.p, state.p, covered.p, cur,
                                              undecided.p + b),
         SVXG_COUNT_LAUNCH());
        (k_mis_cover_claim<<<nblk(n), kT, 0, st>>>(n, A.rowptr, A.col, strong.p, state.p, covered.p, cur, nxt),
         SVXG_COUNT_LAUNCH());
        std::swap(cur, nxt);
      }
      int32_t u = 0;
      TRY(copy_to_host(P, &u, undecided.p + (kBatch - 1), sizeof(int32_t)));
      if (u == 0) break;
      if (u <= kMisTail) {
        // (the long tail of rounds over the few nodes left: one block launch)
        (k_undecided_flags<<<nblk(n), kT, 0, st>>>(n, state.p, flag.p), SVXG_COUNT_LAUNCH());
        int32_t m = 0;
        TRY(exclusive_scan_i32(P, flag.p, rank.p, n, &m));
        (k_list_flagged<<<nblk(n), kT, 0, st>>>(n, flag.p, rank.p, agg1.p), SVXG_COUNT_LAUNCH());
        (k_mis_tail<<<1, 1024, 0, st>>>(agg1.p, m, A.rowptr, A.col, strong.p, state.p, covered.p, cur),
         SVXG_COUNT_LAUNCH());
        break;
      }
    }
    (k_root_flags<<<nblk(n), kT, 0, st>>>(n, state.p, flag.p), SVXG_COUNT_LAUNCH());
    int32_t na1 = 0;
    TRY(exclusive_scan_i32(P, flag.p, rank.p, n, &na1));
    SVXG_CUDA(cudaMemsetAsync(agg1.p, 0xff, sizeof(int32_t) * size_t(n), st));
    (k_agg_pass1<<<nblk(n), kT, 0, st>>>(n, A.rowptr, A.col, strong.p, state.p, rank.p, agg1.p), SVXG_COUNT_LAUNCH());
    (k_agg_pass2<<<nblk(n), kT, 0, st>>>(n, A.rowptr, A.col, fro.p, agg1.p, agg), SVXG_COUNT_LAUNCH());
    (k_pass3_flags<<<nblk(n), kT, 0, st>>>(n, A.rowptr, agg, iso.p, noniso.p), SVXG_COUNT_LAUNCH());
    TRY(exclusive_scan_i32(P, iso.p, isorank.p, n, nullptr));
    const int32_t group = P.seg_n > 0 ? 0 : 1;  // (a batch: isolated leftovers stay single, graphs apart)
    (k_pass3_alloc<<<nblk(n), kT, 0, st>>>(n, iso.p, isorank.p, noniso.p, group, alloc.p, gfirst.p),
     SVXG_COUNT_LAUNCH());
    int32_t nalloc = 0;
    TRY(exclusive_scan_i32(P, alloc.p, allocscan.p, n, &nalloc));
    (k_pass3_assign<<<nblk(n), kT, 0, st>>>(n, na1, iso.p, isorank.p, noniso.p, group, allocscan.p, gfirst.p, agg),
     SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaGetLastError());
    na = na1 + nalloc;
    if (!opt.reaggregate || round == 3 || 2 * int64_t(na) <= n) break;
    theta *= 0.5;
  }
  if (na >= n || double(na) > 0.85 * n) {
    P.mem.release(agg);
    return SVXG_OK;
  }
  P.lv.emplace_back();
  Level& F = P.lv[l];
  Level& C = P.lv[l + 1];
  F.parent = agg;
  C.A.n = na;
  trace_mark(P, "coarsen: aggregated");
  // coarse positions and offsets
  {
    Tmp<int32_t> cnt(st), off(st), cursor(st), members(st);
    TRY(cnt.alloc(size_t(na) + 1));
    TRY(off.alloc(size_t(na) + 1));
    TRY(cursor.alloc(size_t(na) + 1));
    TRY(members.alloc(size_t(n)));
    SVXG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (size_t(na) + 1), st));
    SVXG_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * (size_t(na) + 1), st));
    (k_count_members<<<nblk(n), kT, 0, st>>>(n, agg, cnt.p), SVXG_COUNT_LAUNCH());
    TRY(exclusive_scan_i32(P, cnt.p, off.p, int64_t(na) + 1, nullptr));
    (k_fill_members<<<nblk(n), kT, 0, st>>>(n, agg, off.p, cursor.p, members.p), SVXG_COUNT_LAUNCH());
    TRY(P.mem.alloc(&C.pos, 3 * size_t(na)));
    (k_coarse_pos<<<nblk(na), kT, 0, st>>>(na, off.p, members.p, F.pos, C.pos), SVXG_COUNT_LAUNCH());
  }
  Tmp<double> off3(st);
  TRY(off3.alloc(3 * size_t(n)));
  (k_offsets<<<nblk(n), kT, 0, st>>>(n, agg, F.pos, C.pos, off3.p), SVXG_COUNT_LAUNCH());
  trace_mark(P, "coarsen: positions");
  // prolongation
  double omega = 0.0;
  if (smoothed) {
    double lm = 0.0;
    TRY(estimate_lmax(P, F, &lm));
    trace_mark(P, "coarsen: lmax");
    F.lmax = lm;
    omega = (4.0 / 3.0) / maxd(1e-300, lm);
  }
  {
    const Bsr& A = F.A;
    Tmp<int32_t> plen(st), scratch(st);
    TRY(plen.alloc(size_t(n) + 1));
    TRY(scratch.alloc(size_t(nnzb) + size_t(n) + 1));
    SVXG_CUDA(cudaMemsetAsync(plen.p, 0, sizeof(int32_t) * (size_t(n) + 1), st));
    (k_p_count<<<nblk(n), kT, 0, st>>>(n, A.rowptr, A.col, agg, smoothed ? 1 : 0, plen.p, scratch.p, INT_MAX), SVXG_COUNT_LAUNCH());
    TRY(P.mem.alloc(&F.prow, size_t(n) + 1));
    int32_t pnnz = 0;
    TRY(exclusive_scan_i32(P, plen.p, F.prow, int64_t(n) + 1, &pnnz));
    F.pnnz = pnnz;
    TRY(P.mem.alloc(&F.pcol, size_t(pnnz)));
    TRY(P.mem.alloc(&F.pval, size_t(pnnz) * 36));
    (k_p_values<<<unsigned((n + kPWarps - 1) / kPWarps), 32 * kPWarps, 0, st>>>(n, A.rowptr, A.col, A.val, agg, off3.p, F.dinv, omega, F.prow,
                                              scratch.p, F.pcol, F.pval), SVXG_COUNT_LAUNCH());
  }
  if (smoothed) P.amg_build_work += 12 * nnzb;
  int64_t ap_products = 0;  // (the block products of A P: |P row col(k)| for every block k of A)
  {
    Tmp<unsigned long long> acc(st);
    TRY(acc.alloc(1));
    SVXG_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(unsigned long long), st));
    (k_work_ap<<<nblk(nnzb), kT, 0, st>>>(nnzb, F.A.col, F.prow, acc.p), SVXG_COUNT_LAUNCH());
    unsigned long long w = 0;
    TRY(copy_to_host(P, &w, acc.p, sizeof(w)));
    P.amg_build_work += int64_t(w);
    ap_products = int64_t(w / 6);
  }
  trace_mark(P, "coarsen: prolongation");
  // restriction lists
  {
    Tmp<int32_t> cnt(st), cursor(st), erow(st);
    TRY(cnt.alloc(size_t(na) + 1));
    TRY(cursor.alloc(size_t(na) + 1));
    TRY(erow.alloc(size_t(F.pnnz)));
    SVXG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (size_t(na) + 1), st));
    SVXG_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * (size_t(na) + 1), st));
    (k_r_count<<<nblk(F.pnnz), kT, 0, st>>>(F.pnnz, F.pcol, cnt.p), SVXG_COUNT_LAUNCH());
    TRY(P.mem.alloc(&F.rrow, size_t(na) + 1));
    TRY(exclusive_scan_i32(P, cnt.p, F.rrow, int64_t(na) + 1, nullptr));
    TRY(P.mem.alloc(&F.rent_e, size_t(F.pnnz)));
    TRY(P.mem.alloc(&F.rent_i, size_t(F.pnnz)));
    (k_r_fill<<<nblk(n), kT, 0, st>>>(n, F.prow, F.pcol, F.rrow, cursor.p, F.rent_e), SVXG_COUNT_LAUNCH());
    (k_entry_rows<<<nblk(n), kT, 0, st>>>(n, F.prow, erow.p), SVXG_COUNT_LAUNCH());
    (k_r_sort<<<nblk(na), kT, 0, st>>>(na, F.rrow, F.rent_e, F.rent_i, erow.p), SVXG_COUNT_LAUNCH());
  }
  trace_mark(P, "coarsen: restriction lists");
  // Galerkin: A P
  int64_t apnnz_total = 0;
  Tmp<int32_t> aprow(st), apcol(st);
  Tmp<double> apval(st);
  {
    Tmp<int32_t> bound(st), scratch(st);
    Tmp<int64_t> soff(st);
    TRY(bound.alloc(size_t(n) + 1));
    TRY(soff.alloc(size_t(n) + 1));
    SVXG_CUDA(cudaMemsetAsync(bound.p, 0, sizeof(int32_t) * (size_t(n) + 1), st));
    (k_ap_bound<<<nblk(n), kT, 0, st>>>(n, F.A.rowptr, F.A.col, F.prow, bound.p), SVXG_COUNT_LAUNCH());
    int64_t stotal = 0;
    TRY(offsets64(P, bound.p, n, soff.p, &stotal));
    TRY(scratch.alloc(size_t(stotal) + 1));
    TRY(aprow.alloc(size_t(n) + 1));
    Tmp<int32_t> aplen(st);
    TRY(aplen.alloc(size_t(n) + 1));
    SVXG_CUDA(cudaMemsetAsync(aplen.p, 0, sizeof(int32_t) * (size_t(n) + 1), st));
    if (na <= kBitmapCols)
      (k_ap_count_bitmap<<<unsigned((n + kBitmapWarps - 1) / kBitmapWarps), 32 * kBitmapWarps, 0, st>>>(
           n, na, F.A.rowptr, F.A.col, F.prow, F.pcol, aplen.p, scratch.p, soff.p),
       SVXG_COUNT_LAUNCH());
    else
      (k_ap_count<<<nblk(n), kT, 0, st>>>(n, F.A.rowptr, F.A.col, F.prow, F.pcol, aplen.p, scratch.p, soff.p, INT_MAX),
       SVXG_COUNT_LAUNCH());
    int32_t apnnz = 0;
    TRY(exclusive_scan_i32(P, aplen.p, aprow.p, int64_t(n) + 1, &apnnz));
    apnnz_total = apnnz;
    TRY(apcol.alloc(size_t(apnnz)));
    TRY(apval.alloc(size_t(apnnz) * 36));
    const bool timed = P.timer_on && P.timer_kind == SVXG_TIMER_GALERKIN_AP;
    if (timed) TRY(timer_mark(P));
    if (n < kFewRowsAP) {  // (levels of few rows: a warp per block of A P)
      if (apnnz > 0)
        (k_ap_values_warp<<<unsigned((int64_t(apnnz) + kApWarps - 1) / kApWarps), 32 * kApWarps, 0, st>>>(
             n, int64_t(apnnz), F.A.rowptr, F.A.col, F.A.val, F.prow, F.pcol, F.pval, aprow.p, scratch.p, soff.p,
             apcol.p, apval.p),
         SVXG_COUNT_LAUNCH());
    } else {
      (k_ap_values_acc<<<unsigned((n + kAccWarps - 1) / kAccWarps), 32 * kAccWarps, 0, st>>>(
           n, F.A.rowptr, F.A.col, F.A.val, F.prow, F.pcol, F.pval, aprow.p, scratch.p, soff.p, apcol.p, apval.p),
       SVXG_COUNT_LAUNCH());
    }
    if (timed) {
      TRY(timer_mark(P, true));
      P.timer_work += ap_products;  // (6x6 by 6x6 block products: 432 FP64 operations each, no contraction)
    }
  }
  {
    Tmp<unsigned long long> acc(st);
    TRY(acc.alloc(1));
    SVXG_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(unsigned long long), st));
    (k_work_rap<<<nblk(n), kT, 0, st>>>(n, F.prow, aprow.p, acc.p), SVXG_COUNT_LAUNCH());
    unsigned long long w = 0;
    TRY(copy_to_host(P, &w, acc.p, sizeof(w)));
    P.amg_build_work += int64_t(w);
  }
  trace_mark(P, "coarsen: A P");
  // Galerkin: P^T (A P) by coarse row
  {
    Tmp<int32_t> bound(st), scratch(st), clen(st);
    Tmp<int64_t> soff(st);
    TRY(bound.alloc(size_t(na) + 1));
    TRY(soff.alloc(size_t(na) + 1));
    SVXG_CUDA(cudaMemsetAsync(bound.p, 0, sizeof(int32_t) * (size_t(na) + 1), st));
    (k_c_bound<<<nblk(na), kT, 0, st>>>(na, F.rrow, F.rent_i, aprow.p, bound.p), SVXG_COUNT_LAUNCH());
    int64_t stotal = 0;
    TRY(offsets64(P, bound.p, na, soff.p, &stotal));
    TRY(scratch.alloc(size_t(stotal) + 1));
    TRY(clen.alloc(size_t(na) + 1));
    SVXG_CUDA(cudaMemsetAsync(clen.p, 0, sizeof(int32_t) * (size_t(na) + 1), st));
    if (na <= kBitmapCols)
      (k_c_count_bitmap<<<unsigned((na + kBitmapWarps - 1) / kBitmapWarps), 32 * kBitmapWarps, 0, st>>>(
           na, F.rrow, F.rent_i, aprow.p, apcol.p, clen.p, scratch.p, soff.p),
       SVXG_COUNT_LAUNCH());
    else
      (k_c_count<<<nblk(na), kT, 0, st>>>(na, F.rrow, F.rent_i, aprow.p, apcol.p, clen.p, scratch.p, soff.p, INT_MAX),
       SVXG_COUNT_LAUNCH());
    TRY(P.mem.alloc(&C.A.rowptr, size_t(na) + 1));
    int32_t cnnz = 0;
    TRY(exclusive_scan_i32(P, clen.p, C.A.rowptr, int64_t(na) + 1, &cnnz));
    trace_mark(P, "coarsen: coarse pattern");
    C.A.nnzb = cnnz;
    TRY(P.mem.alloc(&C.A.col, size_t(cnnz)));
    TRY(P.mem.alloc(&C.A.val, size_t(cnnz) * 36));
    const double scale = (!smoothed && opt.coarse_scale != 1.0) ? opt.coarse_scale : 1.0;
    // (levels of few coarse rows: a warp per block of C; wider levels: a warp per coarse row, whose
    // restriction entries are walked once rather than once per block of the row)
    if (na < kFewRows) {
      if (cnnz > 0)
        (k_c_values_warp<<<unsigned((int64_t(cnnz) + kCWarps - 1) / kCWarps), 32 * kCWarps, 0, st>>>(
             na, int64_t(cnnz), F.rrow, F.rent_i, F.rent_e, F.pval, aprow.p, apcol.p, apval.p, C.A.rowptr, scratch.p,
             soff.p, C.A.col, C.A.val, scale),
         SVXG_COUNT_LAUNCH());
    } else if (apnnz_total >= 6 * int64_t(n)) {
      (k_c_values_acc<<<unsigned((na + kAccWarps - 1) / kAccWarps), 32 * kAccWarps, 0, st>>>(
           na, F.rrow, F.rent_i, F.rent_e, F.pval, aprow.p, apcol.p, apval.p, C.A.rowptr, scratch.p, soff.p, C.A.col,
           C.A.val, scale),
       SVXG_COUNT_LAUNCH());
    } else {
      (k_c_values<<<nblk(32 * int64_t(na), 128), 128, 0, st>>>(na, F.rrow, F.rent_i, F.rent_e, F.pval, aprow.p, apcol.p,
                                                                apval.p, C.A.rowptr, scratch.p, soff.p, C.A.col, C.A.val,
                                                                scale),
       SVXG_COUNT_LAUNCH());
    }
  }
  SVXG_CUDA(cudaGetLastError());
  trace_mark(P, "coarsen: coarse values");
  bool fin = false;
  TRY(finalize_level(P, P.lv[l + 1], &fin));
  if (!fin) {
    // (coarse level singular: the reference's coarsen returns false after F's P is made)
    Level& Cx = P.lv.back();
    P.mem.release(Cx.A.rowptr);
    P.mem.release(Cx.A.col);
    P.mem.release(Cx.A.val);
    P.mem.release(Cx.dinv);
    P.mem.release(Cx.pos);
    P.lv.pop_back();
    return SVXG_OK;
  }
  *made = true;
  return SVXG_OK;
}

int factor_coarsest(Problem& P) {
  const Level& L = P.lv.back();
  if (L.A.n > 4 * P.opt.amg.coarse_max) {
    P.chol_n = 0;
    return SVXG_OK;
  }
  const int32_t m = 6 * L.A.n;
  P.chol_n = m;
  P.amg_build_work += int64_t(m) * m * m / 108;
  TRY(P.mem.alloc(&P.d_chol, size_t(m) * size_t(m)));
  cudaStream_t st = P.stream;
  SVXG_CUDA(cudaMemsetAsync(P.d_chol, 0, sizeof(double) * size_t(m) * size_t(m), st));
  (k_dense_fill<<<nblk(36 * int64_t(L.A.n)), kT, 0, st>>>(L.A.n, L.A.rowptr, L.A.col, L.A.val, m, P.d_chol),
   SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  // the factor (in place) and the inverse the cycle applies: dense.cu
  TRY(P.mem.alloc(&P.d_cinv, 2 * size_t(m) * size_t(m)));
  TRY(P.mem.alloc(&P.d_cvec, 2 * size_t(m)));
  return dense_factor_inverse(P, m, P.d_chol, P.d_chol, P.d_cinv);
}

__global__ void k_level0_pos(int32_t n, const svxg_node* nodes, const int32_t* dof, double* pos) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t d = dof[i];
  if (d < 0) return;
  pos[3 * int64_t(d)] = nodes[i].c.x;
  pos[3 * int64_t(d) + 1] = nodes[i].c.y;
  pos[3 * int64_t(d) + 2] = nodes[i].c.z;
}

__global__ void k_state_norm_out(const double* state, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = state[1];
}

}  // namespace

#ifndef SVXG_FAST_SETUP
// sqrt of the sequential sum of squares of n device doubles (the power iteration's norm), by the
// path estimate_lmax takes for a vector of that length
int debug_seq_norm(cudaStream_t st, const double* v, int64_t n, double* out_dev) {
  Tmp<double> state(st);
  NormScratch ns(st);
  TRY(state.alloc(3));
  TRY(ns.alloc(n));
  SVXG_CUDA(cudaMemsetAsync(state.p, 0, 3 * sizeof(double), st));
  TRY(launch_norm(st, n, v, nullptr, state.p, ns));
  (k_state_norm_out<<<1, 32, 0, st>>>(state.p, out_dev), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  SVXG_CUDA(host_wait(st));
  return SVXG_OK;
}

#endif

// Amg::build (amg.cpp:277-318) over K
#ifdef SVXG_FAST_SETUP
int build_hierarchy_fast(Problem& P, int32_t* ok) {
#else
int build_hierarchy(Problem& P, int32_t* ok) {
#endif
  *ok = 0;
  P.lv.clear();
  P.chol_n = 0;
  P.amg_work = 0;
  P.amg_build_work = 0;
  if (P.nfree == 0) {
    *ok = 1;
    return SVXG_OK;
  }
  P.lv.emplace_back();
  {
    Level& L0 = P.lv[0];
    L0.A = P.K;  // (level 0's matrix is K itself: shared, not copied)
    TRY(P.mem.alloc(&L0.pos, 3 * size_t(P.nfree)));
    (k_level0_pos<<<nblk(P.n), kT, 0, P.stream>>>(P.n, P.d_nodes, P.d_dof, L0.pos), SVXG_COUNT_LAUNCH());
    bool fin = false;
    TRY(finalize_level(P, L0, &fin));
    trace_mark(P, "level 0 finalized");
    if (!fin) {
      P.mem.release(L0.pos);
      P.mem.release(L0.dinv);
      P.lv.clear();
      return SVXG_OK;
    }
  }
  const svxg_amg_options& o = P.opt.amg;
  const int max_levels = std::min(o.max_levels, 16);
  while (int(P.lv.size()) < max_levels && P.lv.back().A.n > o.coarse_max) {
    const Bsr& L = P.lv.back().A;
    const bool dense = P.lv.size() > 1 && L.nnzb > 80 * int64_t(L.n);
    if (dense && !o.coarsen_dense) break;
    bool made = false;
    TRY(coarsen(P, P.lv.size() - 1, !dense && o.smoothed, &made));
    trace_mark(P, "level coarsened");
    if (!made) break;
    if (dense) break;
  }
  TRY(factor_coarsest(P));
  trace_mark(P, "coarsest factored");
  // work per apply (amg.cpp:306-316)
  for (size_t l = 0; l < P.lv.size(); ++l) {
    const bool last = l + 1 == P.lv.size();
    const int64_t nd = o.dense_work_per_unknown ? P.chol_n : P.chol_n / 6;
    const int64_t blocks = P.lv[l].A.nnzb;
    const int64_t coarsest = P.chol_n > 0 ? std::max<int64_t>(blocks, 2 * nd * nd) : 8 * 2 * blocks;
    const int64_t per = last ? coarsest : blocks * (4 * o.sweeps + 2);
    int64_t g = 1;
    for (size_t k = 0; k < l; ++k) g *= o.gamma;
    P.amg_work += per * g;
  }
  TRY(prepare_cycle(P));
  SVXG_CUDA(host_wait(P.stream));
  *ok = 1;
  return SVXG_OK;
}

}  // namespace svxg
