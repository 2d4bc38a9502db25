// solve.cu - BSR SpMV and the preconditioned conjugate-gradient sequence on the device.
//
// The sequence is the reference's StressProblem::begin / iterate (core/src/stress/stress.cpp:
// 362-464): the same recurrences, breakdown tests (p.q <= 0, r.z <= 0, non-finite loads) and
// convergence test (||r|| <= rtol ||f||), with the dots as deterministic two-level reductions
// (block partial sums, then the last block to finish sums them in block order: no atomics on
// values, identical run to run). alpha, beta and the flags live on the device; an iteration is
// four launches and never waits for the host:
//   1. q = K p with p.q in the epilogue           -> alpha, breakdown
//   2. x += alpha p, r -= alpha q with r.r        -> convergence
//   3. z = M^-1 r (block-Jacobi: fused with r.z; multigrid: the V-cycle, then r.z)
//   4. p = z + beta p
// Every kernel returns at once when the run is done, so a batch of iterations queued past
// convergence costs only launches.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "problem.cuh"
#include "spmv_row.cuh"

namespace svxg {
namespace {

constexpr int kVecT = 256;    // vector kernels: one thread per free node
constexpr int kSpmvT = 256;   // SpMV: one warp per block row
constexpr int kRowsPerBlock = kSpmvT / 32;

// (never a zero-block grid: kernels return for rows past n)
inline unsigned vec_blocks(int32_t nfree) { return unsigned((std::max(nfree, 1) + kVecT - 1) / kVecT); }
inline unsigned spmv_blocks(int32_t n) { return unsigned((std::max(n, 1) + kRowsPerBlock - 1) / kRowsPerBlock); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

// Sum of one value per thread over the block (fixed tree); valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; ++i) s += sh[i];
  return s;
}

// Writes this block's NV partials; returns true in every thread of the last block to finish,
// after which that block may read all partials.
template <int NV>
__device__ __forceinline__ bool publish(const double* vals, double* partials, unsigned* counter) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    for (int v = 0; v < NV; ++v) partials[size_t(blockIdx.x) * NV + v] = vals[v];
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

// In the last block: the NV totals over all blocks' partials, in block order per thread then a
// fixed tree; valid in thread 0. Resets the counter.
template <int NT, int NV>
__device__ __forceinline__ void gather_totals(const double* partials, unsigned* counter, double* out, double* sh) {
  __threadfence();
  for (int v = 0; v < NV; ++v) {
    double s = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += NT) s += __ldcg(&partials[size_t(b) * NV + v]);
    out[v] = block_sum<NT>(s, sh);
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// ---- SpMV ------------------------------------------------------------------------------------
// One warp per block row; lanes 6g + r (g < 5) take block g of each group of five and its row r:
// six consecutive values of the block (16-byte loads) against the column's x (the same six
// values for the group's six lanes: one broadcast load). The five groups' sums meet in lanes
// 0-5 by shuffles.
template <typename V>
__device__ __forceinline__ double row_dot6(const V* m, const double* x);

template <>
__device__ __forceinline__ double row_dot6<double>(const double* m, const double* x) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(m));
  const double2 b = __ldg(reinterpret_cast<const double2*>(m) + 1);
  const double2 c = __ldg(reinterpret_cast<const double2*>(m) + 2);
  const double2 u = __ldg(reinterpret_cast<const double2*>(x));
  const double2 v = __ldg(reinterpret_cast<const double2*>(x) + 1);
  const double2 w = __ldg(reinterpret_cast<const double2*>(x) + 2);
  return a.x * u.x + a.y * u.y + b.x * v.x + b.y * v.y + c.x * w.x + c.y * w.y;
}

enum Epilogue { kPlain = 0, kDotP = 1 };

template <int EPI, int SCHED>
__global__ void __launch_bounds__(kSpmvT) k_spmv(int32_t n, const int32_t* __restrict__ rowptr,
                                                 const int32_t* __restrict__ col, const double* __restrict__ val,
                                                 const double* __restrict__ x, double* __restrict__ y,
                                                 double* partials, unsigned* counter, PcgScalars* s,
                                                 RowSkip skip) {
  __shared__ double sh[kSpmvT / 32];
  if (s && s->done) return;  // (the product of a running sequence: nothing once it is done)
  int c;
  bool lane_ok;
  const int32_t row = sched_row<SCHED>(kRowsPerBlock, &c, &lane_ok);
  const bool row_ok = row < n && !row_skipped(skip, row);
  const double yr = sched_row_product<SCHED, double, double, double>(row_ok, row, rowptr, col, val, x);
  double dp = 0.0;
  if (row_ok && lane_ok) {
    y[6 * int64_t(row) + c] = yr;
    if (EPI == kDotP) dp = x[6 * int64_t(row) + c] * yr;
  }
  if (EPI == kDotP) {
    const double bs = block_sum<kSpmvT>(dp, sh);
    if (publish<1>(&bs, partials, counter)) {
      double tot;
      gather_totals<kSpmvT, 1>(partials, counter, &tot, sh);
      if (threadIdx.x == 0) {
        s->pq = tot;
        s->iters += 1;
        if (!(tot > 0)) {
          s->breakdown = 1;
          s->done = 1;
        } else {
          s->alpha = s->rz / tot;
        }
      }
    }
  }
}

// The CG product with its fused p.q: each warp takes kDotSteps row steps (the block's warps on
// consecutive warp indices at every step) before the block's reduction, whose FP64 shuffle tree
// and partials counter a block otherwise pays every 8 (or 40) rows - GB300's FP64 pipe bounds
// this kernel, and the counter's wait holds the block's warps.
constexpr int kDotSteps = 4;
template <int SCHED>
__global__ void __launch_bounds__(kSpmvT) k_spmv_dot(int32_t n, const int32_t* __restrict__ rowptr,
                                                     const int32_t* __restrict__ col, const double* __restrict__ val,
                                                     const double* __restrict__ x, double* __restrict__ y,
                                                     double* partials, unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kSpmvT / 32];
  if (s->done) return;
  double dp = 0.0;
  for (int j = 0; j < kDotSteps; ++j) {
    int c;
    bool lane_ok;
    const int32_t warp = (int32_t(blockIdx.x) * kDotSteps + j) * kRowsPerBlock + (threadIdx.x >> 5);
    const int32_t row = sched_row_of<SCHED>(warp, &c, &lane_ok);
    const bool row_ok = row < n;
    if (SCHED == kWarpRow && !row_ok) break;  // (warp-uniform; the warp's rows only grow)
    const double yr = sched_row_product<SCHED, double, double, double>(row_ok, row, rowptr, col, val, x);
    if (row_ok && lane_ok) {
      y[6 * int64_t(row) + c] = yr;
      dp += x[6 * int64_t(row) + c] * yr;
    }
  }
  const double bs = block_sum<kSpmvT>(dp, sh);
  if (publish<1>(&bs, partials, counter)) {
    double tot;
    gather_totals<kSpmvT, 1>(partials, counter, &tot, sh);
    if (threadIdx.x == 0) {
      s->pq = tot;
      s->iters += 1;
      if (!(tot > 0)) {
        s->breakdown = 1;
        s->done = 1;
      } else {
        s->alpha = s->rz / tot;
      }
    }
  }
}

// The CG products over K's row slots (spmv_row.cuh slot_rows_product): warp w of the grid takes
// slots [5 kSlotRows w, 5 kSlotRows (w + 1)), kSlotRows rows a lane group. With EPI == kPlain:
// y = K x alone; kDotP adds p.q, alpha and the breakdown test as k_spmv_dot. (kSlotRows 2 at three
// blocks an SM measured fastest on the city block's K: 109 us, against 112-175 us for 1, 3 and 4
// rows at the occupancies their registers allow, and 126 us for the table schedules.)
#ifndef SVXG_SLOT_ROWS
#define SVXG_SLOT_ROWS 2
#endif
#ifndef SVXG_SLOT_MINBLOCKS
#define SVXG_SLOT_MINBLOCKS 3
#endif
constexpr int kSlotRows = SVXG_SLOT_ROWS;
template <int EPI, bool SKIP = false>
__global__ void __launch_bounds__(kSpmvT, SVXG_SLOT_MINBLOCKS) k_spmv_slots(int32_t n, const int4* __restrict__ slots,
                                                                           const int32_t* __restrict__ col,
                                                                           const double* __restrict__ val,
                                                                           const double* __restrict__ x,
                                                                           double* __restrict__ y, double* partials,
                                                                           unsigned* counter, PcgScalars* s,
                                                                           RowSkip skip) {
  __shared__ double sh[kSpmvT / 32];
  if (s && s->done) return;  // (the product of a running sequence: nothing once it is done)
  const int c = (threadIdx.x & 31) % 6;
  const int64_t first = (int64_t(blockIdx.x) * kRowsPerBlock + (threadIdx.x >> 5)) * (5 * kSlotRows);
  int32_t row[kSlotRows];
  bool ok[kSlotRows];
  double yr[kSlotRows];
  slot_rows_product<kSlotRows, double, double, double, SKIP>(slots, first, n, col, val, x, row, ok, yr, skip);
  double dp = 0.0;
#pragma unroll
  for (int j = 0; j < kSlotRows; ++j)
    if (ok[j]) {
      y[6 * int64_t(row[j]) + c] = yr[j];
      if (EPI == kDotP) dp = fma(x[6 * int64_t(row[j]) + c], yr[j], dp);
    }
  if (EPI == kDotP) {
    const double bs = block_sum<kSpmvT>(dp, sh);
    if (publish<1>(&bs, partials, counter)) {
      double tot;
      gather_totals<kSpmvT, 1>(partials, counter, &tot, sh);
      if (threadIdx.x == 0) {
        s->pq = tot;
        s->iters += 1;
        if (!(tot > 0)) {
          s->breakdown = 1;
          s->done = 1;
        } else {
          s->alpha = s->rz / tot;
        }
      }
    }
  }
}

// skip (EPI kPlain only): rows of stopped graphs of a batch get no product
template <int EPI>
void launch_spmv(cudaStream_t st, int sched, int32_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                 const double* x, double* y, double* partials, unsigned* counter, PcgScalars* s,
                 const int4* slots = nullptr, RowSkip skip = RowSkip{}) {
  if (slots) {
    const int64_t per = int64_t(kRowsPerBlock) * kSlotRows * 5;
    const unsigned g = unsigned((std::max<int64_t>(n, 1) + per - 1) / per);
    if (EPI == kPlain && skip.flag)
      (k_spmv_slots<kPlain, true><<<g, kSpmvT, 0, st>>>(n, slots, col, val, x, y, partials, counter, s, skip),
       SVXG_COUNT_LAUNCH());
    else
      (k_spmv_slots<EPI><<<g, kSpmvT, 0, st>>>(n, slots, col, val, x, y, partials, counter, s, RowSkip{}),
       SVXG_COUNT_LAUNCH());
    return;
  }
  if (EPI == kDotP) {
    const int per = kRowsPerBlock * kDotSteps * (sched == kGroupRow ? 5 : 1);
    const unsigned g = unsigned((std::max(n, 1) + per - 1) / per);
    if (sched == kGroupRow)
      (k_spmv_dot<kGroupRow><<<g, kSpmvT, 0, st>>>(n, rowptr, col, val, x, y, partials, counter, s),
       SVXG_COUNT_LAUNCH());
    else
      (k_spmv_dot<kWarpRow><<<g, kSpmvT, 0, st>>>(n, rowptr, col, val, x, y, partials, counter, s),
       SVXG_COUNT_LAUNCH());
  } else if (sched == kGroupRow) {
    const unsigned g = unsigned((std::max(n, 1) + 5 * kRowsPerBlock - 1) / (5 * kRowsPerBlock));
    (k_spmv<EPI, kGroupRow><<<g, kSpmvT, 0, st>>>(n, rowptr, col, val, x, y, partials, counter, s, skip),
     SVXG_COUNT_LAUNCH());
  } else {
    (k_spmv<EPI, kWarpRow><<<spmv_blocks(n), kSpmvT, 0, st>>>(n, rowptr, col, val, x, y, partials, counter, s,
                                                               skip),
     SVXG_COUNT_LAUNCH());
  }
}

// ---- vector kernels (one thread per free node, 6 entries) ---------------------------------------

// r = f - q, partial f.f (begin)
__global__ void k_begin_r(int32_t nfree, const double* f, const double* q, double* r, double* partials,
                          unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kVecT / 32];
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  double ff = 0.0;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) {
      const double fv = f[6 * int64_t(i) + c];
      r[6 * int64_t(i) + c] = fv - q[6 * int64_t(i) + c];
      ff += fv * fv;
    }
  const double bs = block_sum<kVecT>(ff, sh);
  if (publish<1>(&bs, partials, counter)) {
    double tot;
    gather_totals<kVecT, 1>(partials, counter, &tot, sh);
    if (threadIdx.x == 0) s->bn = sqrt(tot);
  }
}

// zero x and r when the load is zero or not finite (stress.cpp:389-394)
__global__ void k_begin_zero(int32_t nfree, double* x, double* r, const PcgScalars* s) {
  if (s->bn > 0.0) return;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) x[6 * int64_t(i) + c] = r[6 * int64_t(i) + c] = 0.0;
}

// z = Jinv r (block-Jacobi), and r.z; MODE 0: begin (rz, p = z), 1: iteration (beta)
template <int MODE>
__global__ void k_jacobi_rz(int32_t nfree, const double* __restrict__ jinv, const double* __restrict__ r,
                            double* __restrict__ z, double* p, double* partials, unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kVecT / 32];
  if (MODE == 1 && s->done) return;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  double rz = 0.0;
  if (i < nfree) {
    const double* J = jinv + 36 * int64_t(i);
    double rv[6];
    for (int c = 0; c < 6; ++c) rv[c] = r[6 * int64_t(i) + c];
    for (int a = 0; a < 6; ++a) {
      double zv = 0.0;
      for (int c = 0; c < 6; ++c) zv += J[6 * a + c] * rv[c];
      z[6 * int64_t(i) + a] = zv;
      if (MODE == 0) p[6 * int64_t(i) + a] = zv;
      rz += rv[a] * zv;
    }
  }
  const double bs = block_sum<kVecT>(rz, sh);
  if (publish<1>(&bs, partials, counter)) {
    double tot;
    gather_totals<kVecT, 1>(partials, counter, &tot, sh);
    if (threadIdx.x == 0) {
      if (MODE == 0) {
        s->rz = tot;
      } else if (!(tot > 0)) {
        s->breakdown = 1;
        s->done = 1;
      } else {
        s->beta = tot / s->rz;
        s->rz = tot;
      }
    }
  }
}

// r.z after a multigrid preconditioner; MODE 0: begin (rz, p = z), 1: iteration (beta)
template <int MODE>
__global__ void k_rz(int32_t nfree, const double* __restrict__ r, const double* __restrict__ z, double* p,
                     double* partials, unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kVecT / 32];
  if (MODE == 1 && s->done) return;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  double rz = 0.0;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) {
      const double zv = z[6 * int64_t(i) + c];
      rz += r[6 * int64_t(i) + c] * zv;
      if (MODE == 0) p[6 * int64_t(i) + c] = zv;
    }
  const double bs = block_sum<kVecT>(rz, sh);
  if (publish<1>(&bs, partials, counter)) {
    double tot;
    gather_totals<kVecT, 1>(partials, counter, &tot, sh);
    if (threadIdx.x == 0) {
      if (MODE == 0) {
        s->rz = tot;
      } else if (!(tot > 0)) {
        s->breakdown = 1;
        s->done = 1;
      } else {
        s->beta = tot / s->rz;
        s->rz = tot;
      }
    }
  }
}

// the start of iterate(): ||r||, the target, the non-finite and already-converged exits
__global__ void k_iter_start(int32_t nfree, const double* r, double rtol, int32_t maxit, double* partials,
                             unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kVecT / 32];
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  double rr = 0.0;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) {
      const double v = r[6 * int64_t(i) + c];
      rr += v * v;
    }
  const double bs = block_sum<kVecT>(rr, sh);
  if (publish<1>(&bs, partials, counter)) {
    double tot;
    gather_totals<kVecT, 1>(partials, counter, &tot, sh);
    if (threadIdx.x == 0) {
      const double rn = sqrt(tot);
      s->rn = rn;
      s->iters = 0;
      s->converged = 0;
      s->breakdown = 0;
      s->done = 0;
      s->maxit = maxit;
      s->target = rtol * s->bn;
      if (!isfinite(s->bn) || !isfinite(rn)) {
        s->rel_res = INFINITY;
        s->breakdown = 1;
        s->done = 1;
      } else {
        s->rel_res = s->bn > 0 ? rn / s->bn : 0.0;
        if (rn <= s->target || !(s->bn > 0) || nfree == 0 || maxit <= 0) {
          s->converged = (rn <= s->target || !(s->bn > 0) || nfree == 0) ? 1 : 0;
          s->done = 1;
        }
      }
    }
  }
}

// x += alpha p, r -= alpha q, ||r|| and the convergence test
__global__ void k_axpy_rr(int32_t nfree, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                          const double* __restrict__ q, double* partials, unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kVecT / 32];
  if (s->done) return;
  const double alpha = s->alpha;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  double rr = 0.0;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) {
      const int64_t k = 6 * int64_t(i) + c;
      x[k] += alpha * p[k];
      const double rv = r[k] - alpha * q[k];
      r[k] = rv;
      rr += rv * rv;
    }
  const double bs = block_sum<kVecT>(rr, sh);
  if (publish<1>(&bs, partials, counter)) {
    double tot;
    gather_totals<kVecT, 1>(partials, counter, &tot, sh);
    if (threadIdx.x == 0) {
      const double rn = sqrt(tot);
      s->rn = rn;
      s->rel_res = rn / s->bn;
      if (rn <= s->target) {
        s->converged = 1;
        s->done = 1;
      }
    }
  }
}

// p = z + beta p
__global__ void k_p_update(int32_t nfree, const double* __restrict__ z, double* __restrict__ p, PcgScalars* s) {
  if (s->done) return;
  const double beta = s->beta;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) {
      const int64_t k = 6 * int64_t(i) + c;
      p[k] = z[k] + beta * p[k];
    }
}

// the iteration cap ends a call after a full iteration (the sequence resumes in the next call)
__global__ void k_mark_cap(PcgScalars* s) {
  if (threadIdx.x == 0 && !s->done && s->iters >= s->maxit) s->done = 2;
}

// z = Jinv r alone (the preconditioner's application)
__global__ void k_jacobi_apply(int32_t nfree, const double* __restrict__ jinv, const double* __restrict__ r,
                               double* __restrict__ z) {
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= nfree) return;
  const double* J = jinv + 36 * int64_t(i);
  for (int a = 0; a < 6; ++a) {
    double zv = 0.0;
    for (int c = 0; c < 6; ++c) zv += J[6 * a + c] * r[6 * int64_t(i) + c];
    z[6 * int64_t(i) + a] = zv;
  }
}

// ---- a batch: one conjugate-gradient sequence per graph ------------------------------------------
// Graph g of a batch owns free rows [row0[g], row0[g + 1]) (6 entries each), and the batch's
// multigrid couples no two graphs (aggregation keeps them apart), so each graph runs its own
// sequence - its own alpha, beta, breakdown and stopping test, as if it were alone - inside launches
// shared by all. A graph's dots are sums in a fixed order (one block per graph, thread t over
// entries t, t + 256, ..., then a fixed tree): the same bits whatever else the batch holds. The last
// block to finish a reduction sets the run's flags: done when no graph is still running.
// seg (kSegF doubles per graph): ||f||, target, ||r||, r.z, p.q, alpha, beta, iterations at its end,
// and for the error estimate after the solve ||M^-1 r||^2, ||x||^2;
// flag per graph: 0 running, 1 converged, 2 broken down.
constexpr int kSegT = 256;
constexpr int kSegF = 10;
enum SegOp { kSegBn = 0, kSegRz0 = 1, kSegStart = 2, kSegPq = 3, kSegRn = 4, kSegRz = 5, kSegZz = 6, kSegXx = 7 };

template <int OP>
__global__ void __launch_bounds__(kSegT) k_seg_reduce(int32_t nseg, const int32_t* __restrict__ row0,
                                                       const double* __restrict__ a, const double* __restrict__ b,
                                                       double rtol, double* seg, int32_t* flag, double* partials,
                                                       unsigned* counter, PcgScalars* s) {
  __shared__ double sh[kSegT];
  __shared__ bool last;
  if ((OP == kSegPq || OP == kSegRn || OP == kSegRz) && s->done) return;
  const int32_t g = int32_t(blockIdx.x);
  const int64_t e0 = 6 * int64_t(row0[g]), e1 = 6 * int64_t(row0[g + 1]);
  double t = 0.0;
  for (int64_t e = e0 + threadIdx.x; e < e1; e += kSegT) t += a[e] * b[e];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int d = kSegT / 2; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* q = seg + size_t(kSegF) * g;
    const double v = sh[0];
    if (OP == kSegBn) {
      q[0] = sqrt(v);
    } else if (OP == kSegZz) {
      q[8] = v;
    } else if (OP == kSegXx) {
      q[9] = v;
    } else if (OP == kSegRz0) {
      q[3] = v;
    } else if (OP == kSegStart) {
      q[2] = sqrt(v);
      q[1] = rtol * q[0];
      q[7] = 0.0;
      // (a graph without load is there at once, as a solve of zero load is, stress.cpp:389-394)
      flag[g] = (q[0] > 0.0 && !(q[2] <= q[1])) ? 0 : 1;
    } else if (flag[g] == 0) {
      if (OP == kSegPq) {
        q[4] = v;
        if (!(v > 0.0)) {
          flag[g] = 2;
          q[5] = 0.0;
          q[7] = double(s->iters + 1);
        } else {
          q[5] = q[3] / v;
        }
      } else if (OP == kSegRn) {
        q[2] = sqrt(v);
        if (q[2] <= q[1]) {
          flag[g] = 1;
          q[7] = double(s->iters);
        }
      } else {  // kSegRz
        if (!(v > 0.0)) {
          flag[g] = 2;
          q[7] = double(s->iters);
        } else {
          q[6] = v / q[3];
          q[3] = v;
        }
      }
    }
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || OP == kSegBn || OP == kSegRz0 || OP == kSegZz || OP == kSegXx) {
    if (last && threadIdx.x == 0) *counter = 0u;
    return;
  }
  __threadfence();
  // the last block: graphs still running, broken down
  int32_t run = 0, bad = 0;
  for (int32_t k = threadIdx.x; k < nseg; k += kSegT) {
    const int32_t f = __ldcg(&flag[k]);
    run += f == 0;
    bad += f == 2;
  }
  sh[threadIdx.x] = double(run) + 65536.0 * double(bad);
  __syncthreads();
  for (int d = kSegT / 2; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *counter = 0u;
    const int64_t tot = int64_t(sh[0]);
    const int64_t nrun = tot % 65536, nbad = tot / 65536;
    if (OP == kSegPq) s->iters += 1;
    if (OP == kSegStart) {
      if (s->breakdown) return;  // (not finite: the global start already ended the run)
      s->target = -1.0;          // (k_axpy_rr's global test never stops a batch)
      s->converged = nrun == 0 && nbad == 0 ? 1 : 0;
      s->done = nrun == 0 || s->maxit <= 0 ? 1 : 0;
    } else if (nrun == 0) {
      s->converged = nbad == 0 ? 1 : 0;
      s->breakdown = nbad > 0 ? 1 : 0;
      s->done = 1;
    }
  }
}

// x = r = 0 for graphs without load (begin)
__global__ void k_seg_zero(int32_t nf, const int32_t* __restrict__ seg_of_row, const double* __restrict__ seg,
                           double* x, double* r) {
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= nf || seg[size_t(kSegF) * seg_of_row[i]] > 0.0) return;
  for (int c = 0; c < 6; ++c) x[6 * int64_t(i) + c] = r[6 * int64_t(i) + c] = 0.0;
}

// x += alpha_g p, r -= alpha_g q for the rows of graphs still running
__global__ void k_seg_axpy(int32_t nf, const int32_t* __restrict__ seg_of_row, const double* __restrict__ seg,
                           const int32_t* __restrict__ flag, double* __restrict__ x, double* __restrict__ r,
                           const double* __restrict__ p, const double* __restrict__ q, const PcgScalars* s) {
  if (s->done) return;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= nf) return;
  const int32_t g = seg_of_row[i];
  if (flag[g] != 0) return;
  const double alpha = seg[size_t(kSegF) * g + 5];
  for (int c = 0; c < 6; ++c) {
    const int64_t k = 6 * int64_t(i) + c;
    x[k] += alpha * p[k];
    r[k] -= alpha * q[k];
  }
}

// p = z + beta_g p for the rows of graphs still running
__global__ void k_seg_pupdate(int32_t nf, const int32_t* __restrict__ seg_of_row, const double* __restrict__ seg,
                              const int32_t* __restrict__ flag, const double* __restrict__ z, double* __restrict__ p,
                              const PcgScalars* s) {
  if (s->done) return;
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= nf) return;
  const int32_t g = seg_of_row[i];
  if (flag[g] != 0) return;
  const double beta = seg[size_t(kSegF) * g + 6];
  for (int c = 0; c < 6; ++c) {
    const int64_t k = 6 * int64_t(i) + c;
    p[k] = z[k] + beta * p[k];
  }
}

__global__ void k_fill_ones(int32_t nfree, double* x) {
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i < nfree)
    for (int c = 0; c < 6; ++c) x[6 * int64_t(i) + c] = 1.0;
}

// node order <-> free-DOF order
__global__ void k_scatter_free(int32_t n, const int32_t* dof, const double* nodes6, double* free6) {
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= n) return;
  const int32_t d = dof[i];
  if (d < 0) return;
  for (int c = 0; c < 6; ++c) free6[6 * int64_t(d) + c] = nodes6[6 * int64_t(i) + c];
}

__global__ void k_gather_nodes(int32_t n, const int32_t* dof, const double* free6, double* nodes6) {
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= n) return;
  const int32_t d = dof[i];
  for (int c = 0; c < 6; ++c) nodes6[6 * int64_t(i) + c] = d >= 0 ? free6[6 * int64_t(d) + c] : 0.0;
}

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

}  // namespace

// an event before (closing = false) or after a timed launch
int timer_mark(Problem& P, bool closing) {
  const size_t k = 2 * P.timer_used + (closing ? 1 : 0);
  while (P.timer_events.size() <= k) {
    cudaEvent_t e;
    SVXG_CUDA(cudaEventCreate(&e));
    P.timer_events.push_back(e);
  }
  SVXG_CUDA(cudaEventRecord(P.timer_events[k], P.stream));
  if (closing) ++P.timer_used;
  return SVXG_OK;
}

namespace {

int ensure_run(Problem& P) {
  if (P.d_x) return SVXG_OK;
  const size_t m = 6 * size_t(P.nfree);
  TRY(P.mem.alloc(&P.d_x, m));
  TRY(P.mem.alloc(&P.d_r, m));
  TRY(P.mem.alloc(&P.d_z, m));
  TRY(P.mem.alloc(&P.d_p, m));
  TRY(P.mem.alloc(&P.d_q, m));
  TRY(P.mem.alloc(&P.d_f, m));
  TRY(P.mem.alloc(&P.d_s, 1));
  P.partial_blocks = int32_t(std::max(spmv_blocks(P.nfree), vec_blocks(P.nfree))) + 1;
  TRY(P.mem.alloc(&P.d_partials, size_t(P.partial_blocks) * 4));
  TRY(P.mem.alloc(&P.d_counter, 4));
  SVXG_CUDA(cudaMemsetAsync(P.d_counter, 0, 4 * sizeof(unsigned), P.stream));
  SVXG_CUDA(cudaMemsetAsync(P.d_s, 0, sizeof(PcgScalars), P.stream));
  if (!P.h_s) SVXG_CUDA(cudaMallocHost(&P.h_s, sizeof(PcgScalars)));
  return SVXG_OK;
}

}  // namespace

int spmv(Problem& P, const Bsr& A, const double* x, double* y) {
  if (A.n == 0) return SVXG_OK;
  launch_spmv<kPlain>(P.stream, &A == &P.K ? P.sched_k64 : 0, A.n, A.rowptr, A.col, A.val, x, y, nullptr, nullptr,
                      nullptr, &A == &P.K ? P.d_kslots : nullptr);
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// K's FP64 SpMV schedule from the table; with tune timing on, y = K x is also timed with both
// (a warm-up launch each, then three) and logged
// K's block rows in order of length (a stable counting sort; lengths of 63 blocks and more share
// the last class) as slots {row, first block, length} for the slot schedule of the FP64 CG
// products (spmv_row.cuh slot_rows_product); K of fewer than kSortedMinRows rows keeps the table's
// schedules. The slots depend on K's pattern only, so the products' bits stay a fixed function of
// the operator.
int build_row_slots(Problem& P) {
  P.mem.release(P.d_kslots);
  const int32_t n = P.nfree;
  if (n < kSortedMinRows || !P.K.rowptr) return SVXG_OK;
  std::vector<int32_t> rp(size_t(n) + 1);
  std::vector<int4> sl(static_cast<size_t>(n));
  SVXG_CUDA(cudaMemcpyAsync(rp.data(), P.K.rowptr, sizeof(int32_t) * (size_t(n) + 1), cudaMemcpyDeviceToHost,
                            P.stream));
  SVXG_CUDA(host_wait(P.stream));
  constexpr int kClasses = 64;
  int64_t start[kClasses + 1] = {};
  for (int32_t i = 0; i < n; ++i) ++start[std::min(rp[size_t(i) + 1] - rp[size_t(i)], kClasses - 1) + 1];
  for (int k = 0; k < kClasses; ++k) start[k + 1] += start[k];
  for (int32_t i = 0; i < n; ++i) {
    const int32_t len = rp[size_t(i) + 1] - rp[size_t(i)];
    sl[size_t(start[std::min(len, kClasses - 1)]++)] = make_int4(i, rp[size_t(i)], len, 0);
  }
  TRY(P.mem.alloc(&P.d_kslots, size_t(n)));
  SVXG_CUDA(cudaMemcpyAsync(P.d_kslots, sl.data(), sizeof(int4) * size_t(n), cudaMemcpyHostToDevice, P.stream));
  SVXG_CUDA(host_wait(P.stream));  // (sl is freed on return)
  return SVXG_OK;
}

int tune_k64(Problem& P) {
  TRY(build_row_slots(P));
  P.sched_k64 = table_sched(kOpK64, P.nfree, P.K.nnzb);
  if (P.nfree <= 0 || !tune_timing()) return SVXG_OK;
  const size_t m = 6 * size_t(P.nfree);
  double *x = nullptr, *y = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&x), m * sizeof(double), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&y), m * sizeof(double), P.stream));
  SVXG_CUDA(cudaMemsetAsync(x, 0, m * sizeof(double), P.stream));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms[2] = {0, 0};
  for (int sch = 0; sch < 2; ++sch) {
    launch_spmv<kPlain>(P.stream, sch, P.nfree, P.K.rowptr, P.K.col, P.K.val, x, y, nullptr, nullptr, nullptr);
    cudaEventRecord(e0, P.stream);
    for (int r = 0; r < 3; ++r)
      launch_spmv<kPlain>(P.stream, sch, P.nfree, P.K.rowptr, P.K.col, P.K.val, x, y, nullptr, nullptr, nullptr);
    cudaEventRecord(e1, P.stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms[sch], e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(x, P.stream);
  cudaFreeAsync(y, P.stream);
  P.sched_k64 = tune_decide(P, kOpK64, 0, P.nfree, P.K.nnzb, ms[0], ms[1]);
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// A dedicated timing loop of the conjugate-gradient SpMV: `reps` launches of the kernel an
// iteration runs (q = K p with p.q fused, alpha on the device), each one doing its work (scratch
// scalars with done = 0, so none returns early), on K with p = 1; CUDA events on the problem's
// stream around the loop. The run state of the problem is untouched (scratch vectors and scalars).
int time_cg_spmv(Problem& P, int32_t reps, float* ms_per_launch) {
  *ms_per_launch = 0.0f;
  if (P.nfree <= 0 || reps <= 0 || !P.K.val) return SVXG_OK;
  TRY(ensure_run(P));
  const size_t m = 6 * size_t(P.nfree);
  double *x = nullptr, *y = nullptr;
  PcgScalars* s = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&x), m * sizeof(double), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&y), m * sizeof(double), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&s), sizeof(PcgScalars), P.stream));
  SVXG_CUDA(cudaMemsetAsync(s, 0, sizeof(PcgScalars), P.stream));
  (k_fill_ones<<<vec_blocks(P.nfree), kVecT, 0, P.stream>>>(P.nfree, x), SVXG_COUNT_LAUNCH());
  cudaEvent_t e0, e1;
  SVXG_CUDA(cudaEventCreate(&e0));
  SVXG_CUDA(cudaEventCreate(&e1));
  launch_spmv<kDotP>(P.stream, P.sched_k64, P.nfree, P.K.rowptr, P.K.col, P.K.val, x, y, P.d_partials, P.d_counter,
                     s, P.d_kslots);  // (warm-up)
  SVXG_CUDA(cudaEventRecord(e0, P.stream));
  for (int32_t r = 0; r < reps; ++r)
    launch_spmv<kDotP>(P.stream, P.sched_k64, P.nfree, P.K.rowptr, P.K.col, P.K.val, x, y, P.d_partials,
                       P.d_counter, s, P.d_kslots);
  SVXG_CUDA(cudaEventRecord(e1, P.stream));
  int32_t done_iters = -1;
  SVXG_CUDA(cudaMemcpyAsync(&done_iters, &s->iters, sizeof(int32_t), cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(cudaEventSynchronize(e1));
  SVXG_CUDA(cudaStreamSynchronize(P.stream));
  float ms = 0.0f;
  SVXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(x, P.stream);
  cudaFreeAsync(y, P.stream);
  cudaFreeAsync(s, P.stream);
  SVXG_CUDA(cudaGetLastError());
  if (done_iters != reps + 1) {
    // (a launch returned early: p.q <= 0 stopped the scalars - no time is reported)
    set_error("time_cg_spmv: " + std::to_string(done_iters) + " of " + std::to_string(reps + 1) + " launches ran");
    return SVXG_ERR_STATE;
  }
  *ms_per_launch = ms / float(reps);
  return SVXG_OK;
}

int free_run(Problem& P) {
  P.mem.release(P.d_x);
  P.mem.release(P.d_r);
  P.mem.release(P.d_z);
  P.mem.release(P.d_p);
  P.mem.release(P.d_q);
  P.mem.release(P.d_f);
  P.mem.release(P.d_s);
  P.mem.release(P.d_mx);
  {
    void* ms = P.d_ms;
    P.mem.release(ms);
    P.d_ms = nullptr;
  }
  P.mem.release(P.d_partials);
  P.mem.release(P.d_counter);
  P.active = false;
  return SVXG_OK;
}

int precondition(Problem& P, const double* r, double* z) {
  if (P.jacobi_only) {
    if (P.nfree > 0) (k_jacobi_apply<<<vec_blocks(P.nfree), kVecT, 0, P.stream>>>(P.nfree, P.d_jinv, r, z), SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaGetLastError());
    return SVXG_OK;
  }
  return precondition_amg(P, r, z);
}

// StressProblem::begin (stress.cpp:362-401); f, u0: device, node order (u0 may be null)
int pcg_begin(Problem& P, const double* f_nodes, const double* u0_nodes) {
  TRY(ensure_run(P));
  const int32_t nf = P.nfree;
  const size_t m = 6 * size_t(nf);
  cudaStream_t st = P.stream;
  SVXG_CUDA(cudaMemsetAsync(P.d_x, 0, m * sizeof(double), st));
  SVXG_CUDA(cudaMemsetAsync(P.d_s, 0, sizeof(PcgScalars), st));
  const unsigned nb_nodes = unsigned((P.n + kVecT - 1) / kVecT);
  if (P.n > 0) {
    (k_scatter_free<<<nb_nodes, kVecT, 0, st>>>(P.n, P.d_dof, f_nodes, P.d_f), SVXG_COUNT_LAUNCH());
    if (u0_nodes) (k_scatter_free<<<nb_nodes, kVecT, 0, st>>>(P.n, P.d_dof, u0_nodes, P.d_x), SVXG_COUNT_LAUNCH());
  }
  if (nf > 0) {
    TRY(spmv(P, P.K, P.d_x, P.d_q));
    (k_begin_r<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_f, P.d_q, P.d_r, P.d_partials, P.d_counter, P.d_s), SVXG_COUNT_LAUNCH());
    (k_begin_zero<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_x, P.d_r, P.d_s), SVXG_COUNT_LAUNCH());
    if (P.seg_n > 0) {
      // a batch: per graph ||f||, zero-load graphs at rest, z = M r, p = z, r.z
      TRY(seg_launch(P, kSegBn, P.d_f, P.d_f, 0.0));
      (k_seg_zero<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_seg_of_row, P.d_seg, P.d_x, P.d_r), SVXG_COUNT_LAUNCH());
      TRY(precondition(P, P.d_r, P.d_z));
      (k_rz<0><<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_r, P.d_z, P.d_p, P.d_partials, P.d_counter, P.d_s),
       SVXG_COUNT_LAUNCH());
      TRY(seg_launch(P, kSegRz0, P.d_r, P.d_z, 0.0));
    } else if (P.jacobi_only) {
      (k_jacobi_rz<0><<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_jinv, P.d_r, P.d_z, P.d_p, P.d_partials,
                                                       P.d_counter, P.d_s), SVXG_COUNT_LAUNCH());
    } else if (mixed_run(P)) {
      // (the mixed run starts each inner sequence from the FP64 residual)
    } else {
      TRY(precondition_amg(P, P.d_r, P.d_z));
      (k_rz<0><<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_r, P.d_z, P.d_p, P.d_partials, P.d_counter, P.d_s), SVXG_COUNT_LAUNCH());
    }
  }
  SVXG_CUDA(cudaGetLastError());
  P.active = true;
  P.run_iters = 0;
  return SVXG_OK;
}

// A whole block-Jacobi iterate() in one block, for the small problems the reference preconditions
// by their diagonal blocks: each iteration's steps in order (q = K p with p.q and alpha, the x and r
// update with ||r|| and the convergence test, z = Jinv r with r.z and beta, the p update, the cap),
// with the same breakdown and stopping rules and the same device scalars as the launches of
// plain_body; block barriers stand for the kernel boundaries, and the dot products are block
// trees (fixed order).
constexpr int kJacobiBlockT = 1024;
constexpr int32_t kJacobiBlockMax = 4096;

__device__ __forceinline__ double block_tree_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int d = kJacobiBlockT / 2; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  const double t = sh[0];
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kJacobiBlockT) k_jacobi_pcg_block(int32_t nf, const int32_t* __restrict__ rowptr,
                                                                    const int32_t* __restrict__ col,
                                                                    const double* __restrict__ val,
                                                                    const double* __restrict__ jinv, double* x,
                                                                    double* r, double* z, double* p, double* q,
                                                                    PcgScalars* s) {
  __shared__ double sh[kJacobiBlockT];
  const int64_t m = 6 * int64_t(nf);
  for (int32_t guard = 0; guard <= s->maxit; ++guard) {
    __syncthreads();
    if (s->done) break;
    // q = K p, p.q
    double pq = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += kJacobiBlockT) {
      const int32_t i = int32_t(t / 6);
      const int c = int(t % 6);
      double y = 0.0;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
        const double* a = val + 36 * int64_t(k) + 6 * c;
        const double* v = p + 6 * int64_t(col[k]);
        y += a[0] * v[0] + a[1] * v[1] + a[2] * v[2] + a[3] * v[3] + a[4] * v[4] + a[5] * v[5];
      }
      q[t] = y;
      pq += p[t] * y;
    }
    pq = block_tree_sum(pq, sh);
    if (threadIdx.x == 0) {
      s->pq = pq;
      s->iters += 1;
      if (!(pq > 0)) {
        s->breakdown = 1;
        s->done = 1;
      } else {
        s->alpha = s->rz / pq;
      }
    }
    __syncthreads();
    if (s->done) break;
    // x += alpha p, r -= alpha q, ||r||
    const double alpha = s->alpha;
    double rr = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += kJacobiBlockT) {
      x[t] += alpha * p[t];
      const double rv = r[t] - alpha * q[t];
      r[t] = rv;
      rr += rv * rv;
    }
    rr = block_tree_sum(rr, sh);
    if (threadIdx.x == 0) {
      const double rn = sqrt(rr);
      s->rn = rn;
      s->rel_res = rn / s->bn;
      if (rn <= s->target) {
        s->converged = 1;
        s->done = 1;
      }
    }
    __syncthreads();
    if (s->done) break;
    // z = Jinv r, r.z, beta
    double rz = 0.0;
    for (int32_t i = threadIdx.x; i < nf; i += kJacobiBlockT) {
      const double* J = jinv + 36 * int64_t(i);
      double rv[6];
      for (int c = 0; c < 6; ++c) rv[c] = r[6 * int64_t(i) + c];
      for (int a = 0; a < 6; ++a) {
        double zv = 0.0;
        for (int c = 0; c < 6; ++c) zv += J[6 * a + c] * rv[c];
        z[6 * int64_t(i) + a] = zv;
        rz += rv[a] * zv;
      }
    }
    rz = block_tree_sum(rz, sh);
    if (threadIdx.x == 0) {
      if (!(rz > 0)) {
        s->breakdown = 1;
        s->done = 1;
      } else {
        s->beta = rz / s->rz;
        s->rz = rz;
      }
    }
    __syncthreads();
    if (s->done) break;
    // p = z + beta p; the cap
    const double beta = s->beta;
    for (int64_t t = threadIdx.x; t < m; t += kJacobiBlockT) p[t] = z[t] + beta * p[t];
    __syncthreads();
    if (threadIdx.x == 0 && !s->done && s->iters >= s->maxit) s->done = 2;
  }
}

// one iteration of every graph of a batch: q = K p, per graph p.q and alpha, x and r, ||r|| and
// the stopping test, z = M r, r.z and beta, p (the batch's sequences, each as stress.cpp:428-461)
int seg_body(Problem& P) {
  const int32_t nf = P.nfree;
  cudaStream_t st = P.stream;
  // (the rows of graphs whose sequence has stopped: no product, no cycle - their q and z are read
  // by nothing until the next begin recomputes every row)
  RowSkip skip;
  if (seg_skip(P)) {
    skip.gmap = P.d_seg_of_row;
    skip.flag = P.d_seg_flag;
  }
  launch_spmv<kPlain>(st, P.sched_k64, nf, P.K.rowptr, P.K.col, P.K.val, P.d_p, P.d_q, nullptr, nullptr, P.d_s,
                      P.d_kslots, skip);
  TRY(seg_launch(P, kSegPq, P.d_p, P.d_q, 0.0));
  (k_seg_axpy<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_seg_of_row, P.d_seg, P.d_seg_flag, P.d_x, P.d_r, P.d_p,
                                                P.d_q, P.d_s), SVXG_COUNT_LAUNCH());
  TRY(seg_launch(P, kSegRn, P.d_r, P.d_r, 0.0));
  P.skip_flag = P.pc_n == nf ? skip.flag : nullptr;
  const int e = precondition(P, P.d_r, P.d_z);
  P.skip_flag = nullptr;
  TRY(e);
  TRY(seg_launch(P, kSegRz, P.d_r, P.d_z, 0.0));
  (k_seg_pupdate<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_seg_of_row, P.d_seg, P.d_seg_flag, P.d_z, P.d_p, P.d_s),
   SVXG_COUNT_LAUNCH());
  (k_mark_cap<<<1, 32, 0, st>>>(P.d_s), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// one iteration of the sequence (stress.cpp:428-461), enqueued on P.stream
int plain_body(Problem& P) {
  if (P.seg_n > 0) return seg_body(P);
  const int32_t nf = P.nfree;
  cudaStream_t st = P.stream;
  if (P.spmv_timer()) TRY(timer_mark(P));
  launch_spmv<kDotP>(st, P.sched_k64, nf, P.K.rowptr, P.K.col, P.K.val, P.d_p, P.d_q, P.d_partials, P.d_counter,
                     P.d_s, P.d_kslots);
  if (P.spmv_timer()) TRY(timer_mark(P, true));
  (k_axpy_rr<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_x, P.d_r, P.d_p, P.d_q, P.d_partials, P.d_counter, P.d_s),
   SVXG_COUNT_LAUNCH());
  if (P.jacobi_only) {
    (k_jacobi_rz<1><<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_jinv, P.d_r, P.d_z, nullptr, P.d_partials, P.d_counter,
                                                      P.d_s), SVXG_COUNT_LAUNCH());
  } else {
    TRY(precondition_amg(P, P.d_r, P.d_z));
    (k_rz<1><<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_r, P.d_z, nullptr, P.d_partials, P.d_counter, P.d_s),
     SVXG_COUNT_LAUNCH());
  }
  (k_p_update<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_z, P.d_p, P.d_s), SVXG_COUNT_LAUNCH());
  (k_mark_cap<<<1, 32, 0, st>>>(P.d_s), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// Whether a batch's iteration bodies skip the rows of its stopped graphs (SVXG_NO_ROW_SKIP=1:
// never; the running graphs' results are the same bits either way).
bool seg_skip(const Problem& P) {
  static const bool off = std::getenv("SVXG_NO_ROW_SKIP") != nullptr;
  return !off && P.seg_n > 1 && P.d_seg_of_row && P.d_seg_flag;
}

// whole iterate() calls as one graph launch (SVXG_NO_GRAPHS=1: host-driven batches instead)
bool use_graphs() {
  static const bool on = std::getenv("SVXG_NO_GRAPHS") == nullptr;
  return on;
}

// Whether this iterate() runs as the loop graph in `slot`: once built, always; otherwise only
// for a problem large enough (kGraphMinFree free nodes) or iterated once already since its
// assemble. A graph is captured and instantiated per assembled problem, and instantiation is a
// host-side cost that also serializes concurrent problems, so a small problem solved once is
// better served by host-driven batches of launches (the live timer also needs those).
bool loop_graph_worth(const Problem& P, const void* slot) {
  if (!use_graphs() || P.spmv_timer()) return false;
  return slot != nullptr || P.nfree >= kGraphMinFree || P.host_loops > 0;
}

// Restarts the FP64 sequence from the current x (the mixed run's fallback): r = f - K x,
// z = M^-1 r, p = z, as begin() does after its scatter.
int pcg_restart_fp64(Problem& P) {
  const int32_t nf = P.nfree;
  cudaStream_t st = P.stream;
  SVXG_CUDA(cudaMemsetAsync(P.d_s, 0, sizeof(PcgScalars), st));
  if (nf > 0) {
    TRY(spmv(P, P.K, P.d_x, P.d_q));
    (k_begin_r<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_f, P.d_q, P.d_r, P.d_partials, P.d_counter, P.d_s), SVXG_COUNT_LAUNCH());
    (k_begin_zero<<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_x, P.d_r, P.d_s), SVXG_COUNT_LAUNCH());
    TRY(precondition_amg(P, P.d_r, P.d_z));
    (k_rz<0><<<vec_blocks(nf), kVecT, 0, st>>>(nf, P.d_r, P.d_z, P.d_p, P.d_partials, P.d_counter, P.d_s), SVXG_COUNT_LAUNCH());
  }
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// StressProblem::iterate (stress.cpp:403-464)
int pcg_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res) {
  svxg_pcg_result out{};
  if (!P.active) {
    if (res) *res = out;
    return SVXG_OK;
  }
  if (mixed_run(P)) return mixed_iterate(P, maxit, rtol, res);
  return plain_iterate(P, maxit, rtol, res);
}

// the FP64 sequence from its current state, up to maxit iterations
int plain_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res) {
  svxg_pcg_result out{};
  const int32_t nf = P.nfree;
  cudaStream_t st = P.stream;
  P.cycle_stop = &P.d_s->done;
  (k_iter_start<<<vec_blocks(std::max(nf, 1)), kVecT, 0, st>>>(nf, P.d_r, rtol, maxit, P.d_partials, P.d_counter,
                                                             P.d_s), SVXG_COUNT_LAUNCH());
  if (P.seg_n > 0 && nf > 0) TRY(seg_launch(P, kSegStart, P.d_r, P.d_r, rtol));
  SVXG_CUDA(cudaGetLastError());
  SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
  SVXG_CUDA(host_wait(st));
  if (P.h_s->done || nf == 0) {
    // (converged, empty or not finite at the start: no iteration)
  } else if (P.jacobi_only && nf <= kJacobiBlockMax && !P.spmv_timer() && P.seg_n == 0) {
    (k_jacobi_pcg_block<<<1, kJacobiBlockT, 0, st>>>(nf, P.K.rowptr, P.K.col, P.K.val, P.d_jinv, P.d_x, P.d_r, P.d_z,
                                                      P.d_p, P.d_q, P.d_s),
     SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaGetLastError());
    SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
  } else if (block_solve_fits(P)) {
    TRY(block_iterate(P));
    SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
  } else if (loop_graph_worth(P, P.loop_plain)) {
    int64_t per = 0;
    TRY(run_loop(P, P.loop_plain, &P.d_s->done, plain_body, &per));
    SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    add_launches(per * std::max<int64_t>(1, P.h_s->iters));
  } else {
    P.host_loops += 1;
    const size_t timed0 = P.timer_used;
    int32_t queued = 0;
    int32_t batch = 2;
    for (;;) {
      SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
      SVXG_CUDA(host_wait(st));
      if (P.h_s->done || queued >= maxit) break;
      const int32_t todo = std::min(batch, maxit - queued);
      for (int32_t it = 0; it < todo; ++it) TRY(plain_body(P));
      queued += todo;
      batch = std::min(batch * 2, 32);
    }
    // the live timer keeps the SpMV launches that did work: the first `iters` of this call (the
    // bodies queued past convergence return at once and are not SpMV launches)
    if (P.spmv_timer()) P.timer_used = std::min(P.timer_used, timed0 + size_t(std::max(P.h_s->iters, 0)));
  }
  P.cycle_stop = nullptr;
  out.iters = P.h_s->iters;
  out.converged = P.h_s->converged;
  out.breakdown = P.h_s->breakdown;
  out.rel_res = P.h_s->rel_res;
  P.run_iters += out.iters;
  if (out.breakdown && !std::isfinite(out.rel_res)) P.active = false;
  if (res) *res = out;
  return SVXG_OK;
}

// graph of each coarse row from its fine rows' prolongation entries (every entry of a fine row
// names an aggregate of the same graph: a batch's hierarchy is block diagonal)
__global__ void k_coarse_gmap(int32_t n, const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                              const int32_t* __restrict__ fine, int32_t* coarse) {
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  if (i >= n) return;
  const int32_t g = fine[i];
  for (int32_t k = prow[i]; k < prow[i + 1]; ++k) coarse[pcol[k]] = g;
}

// Each level's rows by graph, for the skipping in a batch's iteration bodies (level 0: the free
// rows' graphs; a coarse row: its fine rows'; -1 where no fine row names it, never skipped), and
// the cycle's vectors zeroed: a skipped row keeps its last, finite values, which the coarsest
// dense inverse multiplies by its exact zeros between graphs.
int seg_level_maps(Problem& P) {
  if (P.jacobi_only || P.lv.empty() || P.lv[0].A.n != P.nfree) return SVXG_OK;
  cudaStream_t st = P.stream;
  int64_t tot = 0;
  for (size_t l = 1; l < P.lv.size(); ++l) tot += std::max(P.lv[l].A.n, 0);
  if (tot > 0) {
    TRY(P.mem.alloc(&P.d_seg_lmap, size_t(tot)));
    SVXG_CUDA(cudaMemsetAsync(P.d_seg_lmap, 0xff, sizeof(int32_t) * size_t(tot), st));
  }
  P.lv[0].gmap = P.d_seg_of_row;
  int64_t off = 0;
  for (size_t l = 1; l < P.lv.size(); ++l) {
    int32_t* map = P.d_seg_lmap + off;
    off += std::max(P.lv[l].A.n, 0);
    const Level& F = P.lv[l - 1];
    if (F.A.n > 0 && F.prow && F.pcol)
      (k_coarse_gmap<<<vec_blocks(F.A.n), kVecT, 0, st>>>(F.A.n, F.prow, F.pcol, F.gmap, map), SVXG_COUNT_LAUNCH());
    P.lv[l].gmap = map;
  }
  for (Level& L : P.lv)
    for (float* v : {L.b32, L.x32, L.r32, L.t32, L.u32})
      if (v) SVXG_CUDA(cudaMemsetAsync(v, 0, sizeof(float) * 6 * size_t(std::max(L.A.n, 1)), st));
  if (P.d_cvec && P.chol_n > 0) SVXG_CUDA(cudaMemsetAsync(P.d_cvec, 0, sizeof(double) * 2 * size_t(P.chol_n), st));
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// A batch's free-row offsets and each free row's graph from the DOF numbering (free nodes numbered
// in node order, so graph g's free rows are those of its nodes), and its per-graph state; after each
// assembly.
int seg_prepare(Problem& P) {
  P.mem.release(P.d_seg_row);
  P.mem.release(P.d_seg);
  P.mem.release(P.d_seg_flag);
  P.mem.release(P.d_seg_of_row);
  P.mem.release(P.d_seg_lmap);
  for (Level& L : P.lv) L.gmap = nullptr;
  if (P.seg_n <= 0) return SVXG_OK;
  std::vector<int32_t> row0(size_t(P.seg_n) + 1, 0), of_row(size_t(std::max(P.nfree, 1)), 0);
  int32_t fr = 0;
  for (int32_t g = 0; g < P.seg_n; ++g) {
    row0[size_t(g)] = fr;
    for (int64_t i = P.seg_node[size_t(g)]; i < P.seg_node[size_t(g) + 1]; ++i)
      if (P.h_dof[size_t(i)] >= 0) of_row[size_t(fr++)] = g;
  }
  row0[size_t(P.seg_n)] = fr;
  TRY(P.mem.alloc(&P.d_seg_row, size_t(P.seg_n) + 1));
  TRY(P.mem.alloc(&P.d_seg, size_t(kSegF) * size_t(P.seg_n)));
  TRY(P.mem.alloc(&P.d_seg_flag, size_t(P.seg_n)));
  TRY(P.mem.alloc(&P.d_seg_of_row, of_row.size()));
  SVXG_CUDA(cudaMemcpyAsync(P.d_seg_row, row0.data(), sizeof(int32_t) * row0.size(), cudaMemcpyHostToDevice,
                            P.stream));
  SVXG_CUDA(cudaMemcpyAsync(P.d_seg_of_row, of_row.data(), sizeof(int32_t) * of_row.size(), cudaMemcpyHostToDevice,
                            P.stream));
  SVXG_CUDA(cudaMemsetAsync(P.d_seg, 0, sizeof(double) * size_t(kSegF) * size_t(P.seg_n), P.stream));
  SVXG_CUDA(cudaMemsetAsync(P.d_seg_flag, 0, sizeof(int32_t) * size_t(P.seg_n), P.stream));
  TRY(seg_level_maps(P));
  SVXG_CUDA(host_wait(P.stream));  // (row0 and of_row are freed on return)
  return SVXG_OK;
}

// a reduction over every graph of the batch (one block each), its partials counter the problem's
int seg_launch(Problem& P, int op, const double* a, const double* b, double rtol) {
  const unsigned g = unsigned(P.seg_n);
  unsigned* ctr = P.d_counter + 1;  // (a counter of its own: the global reductions use the first)
  switch (op) {
    case kSegBn:
      (k_seg_reduce<kSegBn><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                        P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
      break;
    case kSegRz0:
      (k_seg_reduce<kSegRz0><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                         P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
      break;
    case kSegStart:
      (k_seg_reduce<kSegStart><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg,
                                                           P.d_seg_flag, P.d_partials, ctr, P.d_s),
       SVXG_COUNT_LAUNCH());
      break;
    case kSegPq:
      (k_seg_reduce<kSegPq><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                        P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
      break;
    case kSegRn:
      (k_seg_reduce<kSegRn><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                        P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
      break;
    case kSegZz:
      (k_seg_reduce<kSegZz><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                        P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
      break;
    case kSegXx:
      (k_seg_reduce<kSegXx><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                        P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
      break;
    default:
      (k_seg_reduce<kSegRz><<<g, kSegT, 0, P.stream>>>(P.seg_n, P.d_seg_row, a, b, rtol, P.d_seg, P.d_seg_flag,
                                                        P.d_partials, ctr, P.d_s), SVXG_COUNT_LAUNCH());
  }
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// per graph of a batch after a solve: ||r_g|| / ||f_g|| (0 without load), whether it met its target,
// and the iterations its sequence ran
int seg_results(Problem& P, double* rel_res, int32_t* converged, int32_t* iters, double* err_est) {
  if (P.seg_n <= 0 || !P.d_seg) return SVXG_ERR_STATE;
  std::vector<double> h(size_t(kSegF) * size_t(P.seg_n));
  std::vector<int32_t> fl(size_t(P.seg_n));
  SVXG_CUDA(cudaMemcpyAsync(h.data(), P.d_seg, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(cudaMemcpyAsync(fl.data(), P.d_seg_flag, sizeof(int32_t) * fl.size(), cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(host_wait(P.stream));
  for (int32_t g = 0; g < P.seg_n; ++g) {
    const double* q = &h[size_t(kSegF) * size_t(g)];
    if (rel_res) rel_res[g] = q[0] > 0.0 ? q[2] / q[0] : 0.0;
    if (converged) converged[g] = fl[size_t(g)] == 1 ? 1 : 0;
    if (iters) iters[g] = fl[size_t(g)] == 0 ? P.h_s->iters : int32_t(q[7]);
    if (err_est) err_est[g] = q[9] > 0.0 ? sqrt(q[8] / q[9]) : 0.0;
  }
  return SVXG_OK;
}

// ||z||^2 and ||x||^2 over the free DOFs (two-level, fixed order)
__global__ void k_norm_pair(int32_t nf, const double* __restrict__ z, const double* __restrict__ x, double* partials,
                            unsigned* counter, double* out) {
  __shared__ double sh[kVecT / 32];
  const int32_t i = blockIdx.x * kVecT + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const double a = z[6 * int64_t(i) + c], b = x[6 * int64_t(i) + c];
      v[0] += a * a;
      v[1] += b * b;
    }
  double bs[2];
  bs[0] = block_sum<kVecT>(v[0], sh);
  bs[1] = block_sum<kVecT>(v[1], sh);
  if (publish<2>(bs, partials, counter)) {
    double tot[2];
    gather_totals<kVecT, 2>(partials, counter, tot, sh);
    if (threadIdx.x == 0) {
      out[0] = tot[0];
      out[1] = tot[1];
    }
  }
}

// The solve's error estimate, ||M^-1 r|| / ||x||: one application of the preconditioner to the
// final residual (the FP64 one: the mixed run's last outer residual, the FP64 sequence's own),
// which a multigrid close to K^-1 maps close to the error x* - x itself. Per graph in a batch.
int error_estimate(Problem& P) {
  P.last_err_est = 0.0;
  if (P.nfree <= 0 || !P.d_x) return SVXG_OK;
  P.cycle_stop = nullptr;
  TRY(precondition(P, P.d_r, P.d_z));
  if (P.seg_n > 0) {
    TRY(seg_launch(P, kSegZz, P.d_z, P.d_z, 0.0));
    TRY(seg_launch(P, kSegXx, P.d_x, P.d_x, 0.0));
    return SVXG_OK;
  }
  double* out = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&out), 2 * sizeof(double), P.stream));
  (k_norm_pair<<<vec_blocks(P.nfree), kVecT, 0, P.stream>>>(P.nfree, P.d_z, P.d_x, P.d_partials, P.d_counter, out),
   SVXG_COUNT_LAUNCH());
  double h[2] = {0.0, 0.0};
  SVXG_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, P.stream));
  cudaFreeAsync(out, P.stream);
  SVXG_CUDA(host_wait(P.stream));
  P.last_err_est = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
  return SVXG_OK;
}

int gather_solution(Problem& P, double* u_nodes) {
  if (P.n == 0) return SVXG_OK;
  if (!P.d_x) {
    SVXG_CUDA(cudaMemsetAsync(u_nodes, 0, 6 * size_t(P.n) * sizeof(double), P.stream));
    return SVXG_OK;
  }
  (k_gather_nodes<<<unsigned((P.n + kVecT - 1) / kVecT), kVecT, 0, P.stream>>>(P.n, P.d_dof, P.d_x, u_nodes), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

}  // namespace svxg
