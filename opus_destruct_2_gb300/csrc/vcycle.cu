// vcycle.cu - the multigrid V-cycle on the device, in single precision as the reference's
// (Amg::make_fast / cycle_f / apply, core/src/solve/amg.cpp:594-731): r (f64) -> f32 at entry,
// one cycle from zero, z (f32 -> f64) at exit; the coarsest level solved densely in f64.
//
// The smoother is the one the reference's options name but its cycle does not implement
// (AmgOptions::sgs = false: block-Jacobi Chebyshev, core/include/svx/solve/amg.hpp:53-55): a
// Chebyshev polynomial in D^-1 A on [lmax / 10, lmax] (lmax: the level's power-iteration bound),
// the same polynomial before and after the coarse correction so the cycle stays symmetric (a
// valid conjugate-gradient preconditioner). Unlike the reference's hybrid Gauss-Seidel it has no
// sequential dependence: every step is one warp-per-block-row SpMV with the D^-1 block of the row
// and the vector updates fused into its epilogue (direction vectors double-buffered; x updated
// one step late so that no kernel reads a neighbour's x while it is being written).
//
// Per level and cycle: pre-smoothing (2 kernels), residual (1), restriction (1, an SpMV over
// P^T stored by coarse row), prolongation (1, an SpMV over P by fine row, accumulating),
// post-smoothing (2).
//
// In a batch's iteration (P.skip_flag set) every kernel skips the rows of the graphs whose
// sequence has stopped (each level's rows carry their graph, Level::gmap): the hierarchy is block
// diagonal, so a running graph's rows read only its own rows, except in the coarsest dense
// inverse, whose entries between graphs are exact zeros (times the skipped rows' earlier, finite
// values). A running graph's z is the same bits with and without the skipping.
#include <algorithm>
#include <cmath>

#include "problem.cuh"
#include "spmv_row.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;
constexpr int kRows = kT / 32;
inline unsigned nblk(int64_t n, int t = kT) { return unsigned(std::max<int64_t>(1, (n + t - 1) / t)); }
inline unsigned rblk(int32_t n) { return unsigned(std::max<int32_t>(1, (n + kRows - 1) / kRows)); }

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

constexpr int kChebDegree = 2;      // smoothing polynomial degree (each side)
constexpr double kChebRatio = 10.0; // lmax / lmin of the smoothed interval
constexpr int kCoarseDegree = 8;    // stalled coarsest level: polynomial degree in place of a solve

__global__ void k_cvt(int64_t m, const double* in, float* out, const int32_t* stop = nullptr,
                      RowSkip skip = RowSkip{}) {
  if (stop && *stop) return;
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m && !row_skipped(skip, int32_t(k / 6))) out[k] = float(in[k]);
}

__global__ void k_widen(int64_t m, const float* in, double* out, const int32_t* stop, RowSkip skip) {
  if (stop && *stop) return;
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m && !row_skipped(skip, int32_t(k / 6))) out[k] = double(in[k]);
}

// R (P^T blocks) in restriction order: R_r = P_{rent_e[r]}^T, row-major
__global__ void k_cvt_transpose(int64_t pnnz, const int32_t* rent_e, const double* pval, float* rval) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= pnnz) return;
  const double* P = pval + 36 * int64_t(rent_e[r]);
  float* R = rval + 36 * r;
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b) R[a * 6 + b] = float(P[b * 6 + a]);
}

// Warp-per-row block product in f32: lanes 6g + c (g < 5) take every fifth block of the row
// and its row c; the row's six sums end in lanes 0-5.
__device__ __forceinline__ float row_block_sum(int32_t k0, int32_t k1, const int32_t* __restrict__ col,
                                               const float* __restrict__ val, const float* __restrict__ x) {
  return warp_row_product<float, float, float>(k0, k1, col, val, x);
}

// (D^-1 v)_c for the row's lane c, v held by the row's six lanes
template <int SCHED>
__device__ __forceinline__ float dinv_row(const float* __restrict__ D, float v, int c, bool act) {
  float s = 0.0f;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const float vq = row_component<SCHED>(v, q);
    if (act) s += __ldg(D + 6 * c + q) * vq;
  }
  return s;
}

enum Mode {
  kY = 0,        // y = A x
  kAcc = 1,      // y += A x
  kStep = 2,     // r = rin - A d; dout = c1 d + c2 D^-1 r; x (= or +=) d [+ dout]
  kResPend = 3,  // r = rin - A d; x += d
  kPostStart = 4 // r = b - A x; dout = D^-1 r / theta
};

struct StepArgs {
  const int32_t* stop;  // nonzero: the run is over, return at once
  RowSkip skip;         // output rows of stopped graphs: no product, nothing written
  const float* rin;  // kStep / kResPend: previous residual; kPostStart: b
  float* r;          // residual out
  float* dout;       // next direction
  float* x;          // the smoothed iterate
  const float* D;    // D^-1 blocks (36 per node)
  float c1, c2;
  int x_init;        // kStep: x = d (the first step from zero)
  int x_last;        // kStep: also add dout (the last step)
};

template <int MODE, int SCHED>
__global__ void __launch_bounds__(kT) k_bsr32(int32_t n, const int32_t* __restrict__ rowptr,
                                              const int32_t* __restrict__ col, const float* __restrict__ val,
                                              const float* __restrict__ v, float* y, StepArgs s) {
  if (s.stop && *s.stop) return;
  int c;
  bool lane_ok;
  const int32_t row = sched_row<SCHED>(kRows, &c, &lane_ok);
  const bool row_ok = row < n && !row_skipped(s.skip, row);
  if (SCHED == kWarpRow && !row_ok) return;  // (whole warps exit together)
  const float av = sched_row_product<SCHED, float, float, float>(row_ok, row, rowptr, col, val, v);
  const bool act = lane_ok && row_ok;
  const int64_t o = 6 * int64_t(row) + c;
  if (MODE == kY) {
    if (act) y[o] = av;
  } else if (MODE == kAcc) {
    if (act) y[o] += av;
  } else if (MODE == kStep) {
    const float rv = act ? s.rin[o] - av : 0.0f;
    const float z = dinv_row<SCHED>(s.D + 36 * int64_t(row_ok ? row : 0), rv, c, act);
    if (act) {
      const float dprev = v[o];
      const float dn = s.c1 * dprev + s.c2 * z;
      s.r[o] = rv;
      s.dout[o] = dn;
      float xv = s.x_init ? dprev : s.x[o] + dprev;
      if (s.x_last) xv += dn;
      s.x[o] = xv;
    }
  } else if (MODE == kResPend) {
    if (act) {
      s.r[o] = s.rin[o] - av;
      s.x[o] += v[o];
    }
  } else if (MODE == kPostStart) {
    const float rv = act ? s.rin[o] - av : 0.0f;
    const float z = dinv_row<SCHED>(s.D + 36 * int64_t(row_ok ? row : 0), rv, c, act);
    if (act) {
      s.r[o] = rv;
      s.dout[o] = s.c2 * z;
    }
  }
}

// launch of a mode with the operator's schedule (grid: one warp per row or per five rows)
template <int MODE>
void bsr32(cudaStream_t st, int sched, int32_t n, const int32_t* rowptr, const int32_t* col, const float* val,
           const float* v, float* y, const StepArgs& s) {
  if (sched == kGroupRow) {
    const unsigned g = unsigned(std::max<int64_t>(1, (int64_t(n) + 5 * kRows - 1) / (5 * kRows)));
    (k_bsr32<MODE, kGroupRow><<<g, kT, 0, st>>>(n, rowptr, col, val, v, y, s), SVXG_COUNT_LAUNCH());
  } else {
    (k_bsr32<MODE, kWarpRow><<<rblk(n), kT, 0, st>>>(n, rowptr, col, val, v, y, s), SVXG_COUNT_LAUNCH());
  }
}

// d = D^-1 b / theta (the first Chebyshev direction from x = 0); one thread per node
__global__ void k_cheb_first(int32_t n, const float* __restrict__ D, const float* __restrict__ b, float inv_theta,
                             float* d, const int32_t* stop, RowSkip skip) {
  if (stop && *stop) return;
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || row_skipped(skip, i)) return;
  const float* Di = D + 36 * int64_t(i);
  float bv[6];
  for (int q = 0; q < 6; ++q) bv[q] = b[6 * int64_t(i) + q];
  for (int c = 0; c < 6; ++c) {
    float s = 0.0f;
    for (int q = 0; q < 6; ++q) s += Di[6 * c + q] * bv[q];
    d[6 * int64_t(i) + c] = s * inv_theta;
  }
}

__global__ void k_add(int64_t m, const float* d, float* x, const int32_t* stop, RowSkip skip) {
  if (stop && *stop) return;
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m && !row_skipped(skip, int32_t(k / 6))) x[k] += d[k];
}

// coarsest level: x = L^-T (L^-1 b) in f64 (warp per row, rows of L^-1 and of L^-T)
__global__ void k_dense_mv(int32_t m, const double* __restrict__ M, const float* __restrict__ b32,
                           const double* __restrict__ b64, double* y64, float* y32, const int32_t* stop,
                           RowSkip skip) {
  if (stop && *stop) return;
  const int lane = threadIdx.x & 31;
  const int32_t row = blockIdx.x * kRows + (threadIdx.x >> 5);
  if (row >= m || row_skipped(skip, row / 6)) return;  // (m: 6 per node; warp-uniform)
  double s = 0.0;
  const double* Mr = M + int64_t(row) * m;
  for (int32_t k = lane; k < m; k += 32) s += Mr[k] * (b32 ? double(b32[k]) : b64[k]);
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if (lane == 0) {
    if (y64) y64[row] = s;
    if (y32) y32[row] = float(s);
  }
}

// power iteration for the smoother's bound where the setup left none (f64, 12 steps)
__global__ void k_pow_step(int32_t n, const double* dinv, const double* w, double* v) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* D = dinv + 36 * int64_t(i);
  for (int c = 0; c < 6; ++c) {
    double s = 0.0;
    for (int q = 0; q < 6; ++q) s += D[6 * c + q] * w[6 * int64_t(i) + q];
    v[6 * int64_t(i) + c] = s;
  }
}

__global__ void k_norm_scale(int64_t m, double* v, double* nrm) {
  // one block: norm, then scale
  __shared__ double sh[kT];
  double s = 0.0;
  for (int64_t k = threadIdx.x; k < m; k += blockDim.x) s += v[k] * v[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int d = blockDim.x / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  const double nv = sqrt(sh[0]);
  if (threadIdx.x == 0) *nrm = nv;
  if (nv > 0)
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) v[k] /= nv;
}

__global__ void k_spmv64(int32_t n, const int32_t* rowptr, const int32_t* col, const double* val, const double* x,
                         double* y) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= 6 * int64_t(n)) return;
  const int32_t i = int32_t(t / 6);
  const int r = int(t % 6);
  double s = 0.0;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    for (int q = 0; q < 6; ++q) s += val[36 * int64_t(k) + 6 * r + q] * x[6 * int64_t(col[k]) + q];
  y[t] = s;
}

__global__ void k_fill_ones(int64_t m, double* v) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m) v[k] = 1.0 + 0.001 * double(k % 7);
}

int power_bound(Problem& P, const Level& L, double* out) {
  const int64_t m = 6 * int64_t(L.A.n);
  double *v = nullptr, *w = nullptr, *nv = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&v), m * sizeof(double), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&w), m * sizeof(double), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&nv), sizeof(double), P.stream));
  (k_fill_ones<<<nblk(m), kT, 0, P.stream>>>(m, v), SVXG_COUNT_LAUNCH());
  for (int it = 0; it < 12; ++it) {
    (k_spmv64<<<nblk(m), kT, 0, P.stream>>>(L.A.n, L.A.rowptr, L.A.col, L.A.val, v, w), SVXG_COUNT_LAUNCH());
    (k_pow_step<<<nblk(L.A.n), kT, 0, P.stream>>>(L.A.n, L.dinv, w, v), SVXG_COUNT_LAUNCH());
    (k_norm_scale<<<1, kT, 0, P.stream>>>(m, v, nv), SVXG_COUNT_LAUNCH());
  }
  double h = 0.0;
  cudaMemcpyAsync(&h, nv, sizeof(double), cudaMemcpyDeviceToHost, P.stream);
  cudaFreeAsync(v, P.stream);
  cudaFreeAsync(w, P.stream);
  cudaFreeAsync(nv, P.stream);
  SVXG_CUDA(host_wait(P.stream));
  *out = 1.1 * h;
  return SVXG_OK;
}

// Chebyshev coefficients on [lmax / ratio, lmax] (Saad, Iterative Methods, Alg. 12.1)
struct Cheb {
  float inv_theta;
  float c1[16], c2[16];
};

Cheb chebyshev(double lmax, double ratio, int degree) {
  Cheb C{};
  const double lmin = lmax / ratio;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  C.inv_theta = float(1.0 / theta);
  for (int i = 1; i < degree && i < 16; ++i) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    C.c1[i] = float(rn * rho);
    C.c2[i] = float(2.0 * rn / delta);
    rho = rn;
  }
  return C;
}

// the rows of stopped graphs a level's kernels skip (none outside a batch's iteration)
RowSkip level_skip(const Problem& P, const Level& L) {
  RowSkip k;
  if (P.skip_flag && L.gmap) {
    k.gmap = L.gmap;
    k.flag = P.skip_flag;
  }
  return k;
}

// Chebyshev smoothing of A x = b. from_zero: x = p(D^-1 A) D^-1 b; else x += p(D^-1 A) D^-1 (b - A x).
// Leaves r = b - A x (from_zero, want_residual) for the restriction.
int smooth(Problem& P, const Level& L, const float* b, float* x, bool from_zero, int degree, double ratio,
           bool want_residual) {
  cudaStream_t st = P.stream;
  const int32_t n = L.A.n;
  const Cheb C = chebyshev(L.cheb_lmax, ratio, degree);
  float* d0 = L.t32;
  float* d1 = L.u32;
  StepArgs s{};
  s.stop = P.cycle_stop;
  s.skip = level_skip(P, L);
  s.D = L.dinv32;
  if (from_zero) {
    (k_cheb_first<<<nblk(n), kT, 0, st>>>(n, L.dinv32, b, C.inv_theta, d0, P.cycle_stop, s.skip),
     SVXG_COUNT_LAUNCH());
    s.rin = b;
  } else {
    s.rin = b;
    s.r = L.r32;
    s.dout = d0;
    s.c2 = C.inv_theta;
    bsr32<kPostStart>(st, L.sched_a, n, L.A.rowptr, L.A.col, L.A.val32, x, nullptr, s);
    s.rin = L.r32;
  }
  for (int i = 1; i < degree; ++i) {
    s.r = L.r32;
    s.dout = d1;
    s.x = x;
    s.c1 = C.c1[i];
    s.c2 = C.c2[i];
    s.x_init = (from_zero && i == 1) ? 1 : 0;
    s.x_last = (i == degree - 1 && !(from_zero && want_residual)) ? 1 : 0;
    bsr32<kStep>(st, L.sched_a, n, L.A.rowptr, L.A.col, L.A.val32, d0, nullptr, s);
    s.rin = L.r32;
    std::swap(d0, d1);
  }
  if (from_zero && want_residual) {
    // r = r - A d; x += d (the last direction)
    s.r = L.r32;
    s.x = x;
    if (degree == 1) {
      SVXG_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * 6 * size_t(n), st));
    }
    bsr32<kResPend>(st, L.sched_a, n, L.A.rowptr, L.A.col, L.A.val32, d0, nullptr, s);
  } else if (degree == 1) {
    if (from_zero) {
      SVXG_CUDA(cudaMemcpyAsync(x, d0, sizeof(float) * 6 * size_t(n), cudaMemcpyDeviceToDevice, st));
    } else {
      (k_add<<<nblk(6 * int64_t(n)), kT, 0, st>>>(6 * int64_t(n), d0, x, P.cycle_stop, s.skip), SVXG_COUNT_LAUNCH());
    }
  }
  return SVXG_OK;
}

int cycle(Problem& P, size_t l, const float* b, float* x) {
  cudaStream_t st = P.stream;
  const Level& L = P.lv[l];
  const int32_t n = L.A.n;
  if (l + 1 == P.lv.size()) {
    if (P.chol_n > 0) {
      const int32_t m = P.chol_n;
      const RowSkip sk = level_skip(P, L);
      (k_dense_mv<<<rblk(m), kT, 0, st>>>(m, P.d_cinv, b, nullptr, P.d_cvec, nullptr, P.cycle_stop, sk),
       SVXG_COUNT_LAUNCH());
      (k_dense_mv<<<rblk(m), kT, 0, st>>>(m, P.d_cinv + int64_t(m) * m, nullptr, P.d_cvec, nullptr, x, P.cycle_stop,
                                          sk),
       SVXG_COUNT_LAUNCH());
      return SVXG_OK;
    }
    return smooth(P, L, b, x, true, kCoarseDegree, 30.0, false);
  }
  TRY(smooth(P, L, b, x, true, kChebDegree, kChebRatio, true));
  const Level& C = P.lv[l + 1];
  StepArgs coarse{}, fine{};
  coarse.stop = fine.stop = P.cycle_stop;
  coarse.skip = level_skip(P, C);
  fine.skip = level_skip(P, L);
  // restriction: bc = P^T r
  bsr32<kY>(st, L.sched_r, C.A.n, L.rrow, L.rent_i, L.pval32 + 36 * L.pnnz, L.r32, C.b32, coarse);
  TRY(cycle(P, l + 1, C.b32, C.x32));
  // prolongation: x += P xc
  bsr32<kAcc>(st, L.sched_p, n, L.prow, L.pcol, L.pval32, C.x32, x, fine);
  TRY(smooth(P, L, b, x, false, kChebDegree, kChebRatio, false));
  return SVXG_OK;
}

// the table's schedule for y = A x (n block rows, `blocks` blocks); with tune timing on, both
// schedules are also timed (a launch each to warm, then three) and logged
int tune_bsr32(Problem& P, int kind, int level, int64_t blocks, cudaStream_t st, int32_t n, const int32_t* rowptr,
               const int32_t* col, const float* val, const float* x, float* y) {
  if (n <= 0 || !tune_timing()) return table_sched(kind, n, blocks);
  StepArgs none{};
  cudaEvent_t e[3];
  for (auto& ev : e) cudaEventCreate(&ev);
  float ms[2] = {0, 0};
  for (int sch = 0; sch < 2; ++sch) {
    bsr32<kY>(st, sch, n, rowptr, col, val, x, y, none);
    cudaEventRecord(e[0], st);
    for (int r = 0; r < 3; ++r) bsr32<kY>(st, sch, n, rowptr, col, val, x, y, none);
    cudaEventRecord(e[1], st);
    cudaEventSynchronize(e[1]);
    cudaEventElapsedTime(&ms[sch], e[0], e[1]);
  }
  for (auto& ev : e) cudaEventDestroy(ev);
  return tune_decide(P, kind, level, n, blocks, ms[0], ms[1]);
}

}  // namespace

int prepare_cycle(Problem& P) {
  cudaStream_t st = P.stream;
  for (size_t l = 0; l < P.lv.size(); ++l) {
    Level& L = P.lv[l];
    const int32_t n = L.A.n;
    if (!L.A.val32) {
      TRY(P.mem.alloc(&L.A.val32, 36 * size_t(L.A.nnzb)));
      (k_cvt<<<nblk(36 * L.A.nnzb), kT, 0, st>>>(36 * L.A.nnzb, L.A.val, L.A.val32), SVXG_COUNT_LAUNCH());
      if (l == 0) P.K.val32 = L.A.val32;
    }
    TRY(P.mem.alloc(&L.dinv32, 36 * size_t(n)));
    (k_cvt<<<nblk(36 * int64_t(n)), kT, 0, st>>>(36 * int64_t(n), L.dinv, L.dinv32), SVXG_COUNT_LAUNCH());
    if (L.pnnz > 0 && l + 1 < P.lv.size()) {
      // P blocks by fine row, then P^T blocks in restriction order
      TRY(P.mem.alloc(&L.pval32, 72 * size_t(L.pnnz)));
      (k_cvt<<<nblk(36 * L.pnnz), kT, 0, st>>>(36 * L.pnnz, L.pval, L.pval32), SVXG_COUNT_LAUNCH());
      (k_cvt_transpose<<<nblk(L.pnnz), kT, 0, st>>>(L.pnnz, L.rent_e, L.pval, L.pval32 + 36 * L.pnnz), SVXG_COUNT_LAUNCH());
    }
    for (float** v : {&L.b32, &L.x32, &L.r32, &L.t32, &L.u32}) TRY(P.mem.alloc(v, 6 * size_t(std::max(n, 1))));
    // the schedule of each of the level's operators
    SVXG_CUDA(cudaMemsetAsync(L.t32, 0, sizeof(float) * 6 * size_t(std::max(n, 1)), st));
    L.sched_a = tune_bsr32(P, kOpA32, int(l), L.A.nnzb, st, n, L.A.rowptr, L.A.col, L.A.val32, L.t32, L.u32);
    const bool last = l + 1 == P.lv.size();
    if (!last || P.chol_n == 0) {
      if (L.lmax > 0) L.cheb_lmax = L.lmax;
      else TRY(power_bound(P, L, &L.cheb_lmax));
    }
  }
  for (size_t l = 0; l + 1 < P.lv.size(); ++l) {
    Level& L = P.lv[l];
    const Level& C = P.lv[l + 1];
    L.sched_p = tune_bsr32(P, kOpP32, int(l), L.pnnz, st, L.A.n, L.prow, L.pcol, L.pval32, C.t32, L.u32);
    L.sched_r = tune_bsr32(P, kOpR32, int(l), L.pnnz, st, C.A.n, L.rrow, L.rent_i, L.pval32 + 36 * L.pnnz, L.t32,
                           C.u32);
  }
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// z = M^-1 r: one V-cycle from zero (Amg::apply)
int vcycle(Problem& P, const double* r, double* z) {
  if (P.lv.empty()) return SVXG_OK;
  cudaStream_t st = P.stream;
  Level& L0 = P.lv[0];
  const int64_t m = 6 * int64_t(L0.A.n);
  const RowSkip sk = level_skip(P, L0);
  (k_cvt<<<nblk(m), kT, 0, st>>>(m, r, L0.b32, P.cycle_stop, sk), SVXG_COUNT_LAUNCH());
  TRY(cycle(P, 0, L0.b32, L0.x32));
  (k_widen<<<nblk(m), kT, 0, st>>>(m, L0.x32, z, P.cycle_stop, sk), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// the same on f32 vectors (the mixed-precision inner solve): z = M^-1 r
int vcycle32(Problem& P, const float* r, float* z) {
  if (P.lv.empty()) return SVXG_OK;
  TRY(cycle(P, 0, r, z));
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

}  // namespace svxg
