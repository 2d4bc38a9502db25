// mixed.cu - the mixed-precision solve: FP32 K and FP32 V-cycle inside FP64 iterative refinement.
//
// One AMG-preconditioned CG sequence runs in FP32 (SpMV on K32 = K rounded to f32, the f32
// V-cycle, f32 vectors, dots accumulated in FP64), and the refinement is done by reliable updates
// (Sleijpen & van der Vorst, "Reliable updated residuals in hybrid Bi-CG methods", Computing 56,
// 1996; the scheme mixed-precision lattice solvers use): the iterate is x (FP64) + d (f32); when
// the recurrence residual has fallen by kDelta since the last update, or reached the target,
// d is folded into x and the residual is replaced by the true one, r = f - K x in FP64 (K in FP64).
// The sequence is not restarted, so it keeps the Krylov space and converges like the FP64 CG; it
// stops only on the FP64 residual, so the result meets the same rtol as the plain solve.
// FP64 stays where the benchmark spec keeps it: the residual recomputation, the dots and the coarsest
// dense factor.
#include <cmath>

#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;
constexpr int kRows = kT / 32;
inline unsigned vblk(int32_t n) { return unsigned((std::max(n, 1) + kT - 1) / kT); }
inline unsigned rblk(int32_t n) { return unsigned((std::max(n, 1) + kRows - 1) / kRows); }

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

struct MixedScalars {
  double rz, pq, alpha, beta, rn, rmax, target, bn, rr, rel_res;
  int32_t iters, done, breakdown, update, converged, maxit;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < int(blockDim.x) / 32; ++i) s += sh[i];
  return s;
}

// last-block reduction (as solve.cu): true in every thread of the last block, total in tot
__device__ __forceinline__ bool reduce_last(double v, double* partials, unsigned* counter, double* tot) {
  __shared__ double sh[32];
  __shared__ bool last;
  const double bs = block_sum(v, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = bs;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += __ldcg(&partials[b]);
  const double t = block_sum(s, sh);
  if (threadIdx.x == 0) {
    *tot = t;
    *counter = 0u;
  }
  return true;
}

// y32 = K32 p32 (warp per row), p.y accumulated in f64 -> alpha
__global__ void __launch_bounds__(kT) k_spmv32_dot(int32_t n, const int32_t* __restrict__ rowptr,
                                                   const int32_t* __restrict__ col, const float* __restrict__ val,
                                                   const float* __restrict__ p, float* __restrict__ q,
                                                   double* partials, unsigned* counter, MixedScalars* s) {
  if (s->done) return;
  const int lane = threadIdx.x & 31;
  const int32_t row = blockIdx.x * kRows + (threadIdx.x >> 5);
  const int g = lane / 6, c = lane - 6 * (lane / 6);
  float acc = 0.0f;
  if (row < n && g < 5) {
    const int32_t k1 = rowptr[row + 1];
    for (int32_t k = rowptr[row] + g; k < k1; k += 5) {
      const float2* m = reinterpret_cast<const float2*>(val + 36 * int64_t(k) + 6 * c);
      const float2* xv = reinterpret_cast<const float2*>(p + 6 * int64_t(__ldg(col + k)));
      const float2 a = __ldg(m), b = __ldg(m + 1), d = __ldg(m + 2);
      const float2 u = __ldg(xv), v = __ldg(xv + 1), w = __ldg(xv + 2);
      acc += a.x * u.x + a.y * u.y + b.x * v.x + b.y * v.y + d.x * w.x + d.y * w.y;
    }
  }
  const float a1 = __shfl_sync(0xffffffffu, acc, (c + 6) & 31);
  const float a2 = __shfl_sync(0xffffffffu, acc, (c + 12) & 31);
  const float a3 = __shfl_sync(0xffffffffu, acc, (c + 18) & 31);
  const float a4 = __shfl_sync(0xffffffffu, acc, (c + 24) & 31);
  const float y = acc + a1 + a2 + a3 + a4;
  double dp = 0.0;
  if (row < n && lane < 6) {
    q[6 * int64_t(row) + lane] = y;
    dp = double(p[6 * int64_t(row) + lane]) * double(y);
  }
  double tot;
  if (reduce_last(dp, partials, counter, &tot) && threadIdx.x == 0) {
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

// d += alpha p, r -= alpha q (f32), ||r|| in f64; asks for a reliable update when ||r|| fell by
// kDelta since the last one or reached the target
constexpr double kDelta = 0.1;

__global__ void k_axpy32(int32_t nf, float* __restrict__ d, float* __restrict__ r, const float* __restrict__ p,
                         const float* __restrict__ q, double* partials, unsigned* counter, MixedScalars* s) {
  if (s->done) return;
  const float a = float(s->alpha);
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  double rr = 0.0;
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const int64_t k = 6 * i + c;
      d[k] += a * p[k];
      const float rv = r[k] - a * q[k];
      r[k] = rv;
      rr += double(rv) * double(rv);
    }
  double tot;
  if (reduce_last(rr, partials, counter, &tot) && threadIdx.x == 0) {
    s->rn = sqrt(tot);
    if (s->rn <= s->target || s->rn <= kDelta * s->rmax || !isfinite(s->rn)) s->update = 1;
  }
}

// reliable update, 1/3: x += d, d = 0 (only when asked)
__global__ void k_fold(int32_t nf, double* __restrict__ x, float* __restrict__ d, const MixedScalars* s, int force) {
  if (!(force || (s->update && !s->done))) return;
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      x[6 * i + c] += double(d[6 * i + c]);
      d[6 * i + c] = 0.0f;
    }
}

// reliable update, 2/3: q64 = K x (FP64), warp per row (only when asked)
__global__ void __launch_bounds__(kT) k_spmv64_if(int32_t n, const int32_t* __restrict__ rowptr,
                                                  const int32_t* __restrict__ col, const double* __restrict__ val,
                                                  const double* __restrict__ x, double* __restrict__ y,
                                                  const MixedScalars* s, int force) {
  if (!(force || (s->update && !s->done))) return;
  const int lane = threadIdx.x & 31;
  const int32_t row = blockIdx.x * kRows + (threadIdx.x >> 5);
  const int g = lane / 6, c = lane - 6 * (lane / 6);
  double acc = 0.0;
  if (row < n && g < 5) {
    const int32_t k1 = rowptr[row + 1];
    for (int32_t k = rowptr[row] + g; k < k1; k += 5) {
      const double2* m = reinterpret_cast<const double2*>(val + 36 * int64_t(k) + 6 * c);
      const double2* xv = reinterpret_cast<const double2*>(x + 6 * int64_t(__ldg(col + k)));
      const double2 a = __ldg(m), b = __ldg(m + 1), e = __ldg(m + 2);
      const double2 u = __ldg(xv), v = __ldg(xv + 1), w = __ldg(xv + 2);
      acc += a.x * u.x + a.y * u.y + b.x * v.x + b.y * v.y + e.x * w.x + e.y * w.y;
    }
  }
  const double a1 = __shfl_sync(0xffffffffu, acc, (c + 6) & 31);
  const double a2 = __shfl_sync(0xffffffffu, acc, (c + 12) & 31);
  const double a3 = __shfl_sync(0xffffffffu, acc, (c + 18) & 31);
  const double a4 = __shfl_sync(0xffffffffu, acc, (c + 24) & 31);
  if (row < n && lane < 6) y[6 * int64_t(row) + lane] = acc + a1 + a2 + a3 + a4;
}

// reliable update, 3/3: r = f - q64 in FP64 -> r32; the true ||r|| decides convergence
__global__ void k_true_resid(int32_t nf, const double* __restrict__ f, const double* __restrict__ q,
                             float* __restrict__ r32, double* partials, unsigned* counter, MixedScalars* s,
                             int force) {
  if (!(force || (s->update && !s->done))) return;
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  double rr = 0.0;
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const int64_t k = 6 * i + c;
      const double rv = f[k] - q[k];
      r32[k] = float(rv);
      rr += rv * rv;
    }
  double tot;
  if (reduce_last(rr, partials, counter, &tot) && threadIdx.x == 0) {
    const double rn = sqrt(tot);
    s->rr = tot;
    s->rn = rn;
    s->rmax = rn;
    s->update = 0;
    s->rel_res = s->bn > 0 ? rn / s->bn : 0.0;
    if (!isfinite(rn)) {
      s->breakdown = 1;
      s->done = 1;
    } else if (rn <= s->target) {
      s->converged = 1;
      s->done = 1;
    }
  }
}

// r.z (f64 accumulation); MODE 0: start (rz, p = z), 1: iteration (beta; the cap)
template <int MODE>
__global__ void k_rz32(int32_t nf, const float* __restrict__ r, const float* __restrict__ z, float* p, double* partials,
                       unsigned* counter, MixedScalars* s) {
  if (s->done) return;
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  double rz = 0.0;
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const float zv = z[6 * i + c];
      rz += double(r[6 * i + c]) * double(zv);
      if (MODE == 0) p[6 * i + c] = zv;
    }
  double tot;
  if (reduce_last(rz, partials, counter, &tot) && threadIdx.x == 0) {
    if (!(tot > 0)) {
      s->breakdown = 1;
      s->done = 1;
    } else if (MODE == 0) {
      s->rz = tot;
    } else {
      s->beta = tot / s->rz;
      s->rz = tot;
    }
  }
}

__global__ void k_p32(int32_t nf, const float* __restrict__ z, float* __restrict__ p, const MixedScalars* s) {
  if (s->done) return;
  const float b = float(s->beta);
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  if (i < nf)
    for (int c = 0; c < 6; ++c) p[6 * i + c] = z[6 * i + c] + b * p[6 * i + c];
}

// the iteration cap ends a call after a full iteration (done = 3: the next call resumes)
__global__ void k_cap32(MixedScalars* s) {
  if (threadIdx.x == 0 && !s->done && s->iters >= s->maxit) s->done = 3;
}

// the iteration cap ended a call: the next call resumes (done 3 -> 0)
__global__ void k_resume(MixedScalars* s, double target, int32_t maxit) {
  if (threadIdx.x) return;
  if (s->done == 3) s->done = 0;
  s->iters = 0;
  s->maxit = maxit;
  s->target = target;
  s->converged = 0;
}

int ensure_mixed(Problem& P) {
  const size_t m = 6 * size_t(std::max(P.nfree, 1));
  if (P.d_mx) return SVXG_OK;
  TRY(P.mem.alloc(&P.d_mx, 5 * m));  // d, r32, z32, p32, q32
  MixedScalars* ms = nullptr;
  TRY(P.mem.alloc(&ms, 1));
  P.d_ms = ms;
  if (!P.h_ms) SVXG_CUDA(cudaMallocHost(&P.h_ms, sizeof(MixedScalars)));
  return SVXG_OK;
}

}  // namespace

// begin() of the mixed run, after pcg_begin's FP64 r = f - K x0 and ||f||: r32, d = 0,
// z = M^-1 r32, p = z, r.z
int mixed_begin(Problem& P) {
  TRY(ensure_mixed(P));
  const int32_t nf = P.nfree;
  const size_t m = 6 * size_t(std::max(nf, 1));
  cudaStream_t st = P.stream;
  float* d = P.d_mx;
  float* r32 = d + m;
  float* z32 = d + 2 * m;
  float* p32 = d + 3 * m;
  MixedScalars* s = static_cast<MixedScalars*>(P.d_ms);
  SVXG_CUDA(cudaMemsetAsync(s, 0, sizeof(MixedScalars), st));
  SVXG_CUDA(cudaMemsetAsync(d, 0, sizeof(float) * m, st));
  // ||f|| comes from pcg_begin's scalars; the true residual of x0 with force = 1
  SVXG_CUDA(cudaMemcpyAsync(&s->bn, &P.d_s->bn, sizeof(double), cudaMemcpyDeviceToDevice, st));
  (k_spmv64_if<<<rblk(nf), kT, 0, st>>>(nf, P.K.rowptr, P.K.col, P.K.val, P.d_x, P.d_q, s, 1), SVXG_COUNT_LAUNCH());
  (k_true_resid<<<vblk(nf), kT, 0, st>>>(nf, P.d_f, P.d_q, r32, P.d_partials, P.d_counter, s, 1), SVXG_COUNT_LAUNCH());
  P.cycle_stop = &s->done;
  TRY(vcycle32(P, r32, z32));
  (k_rz32<0><<<vblk(nf), kT, 0, st>>>(nf, r32, z32, p32, P.d_partials, P.d_counter, s), SVXG_COUNT_LAUNCH());
  P.cycle_stop = nullptr;
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// iterate() of the mixed run (stress.cpp:403-464's contract: maxit iterations at most, rtol on
// the FP64 residual, breakdown on p.q <= 0 or r.z <= 0 or a non-finite residual)
int mixed_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res) {
  svxg_pcg_result out{};
  TRY(ensure_mixed(P));
  const int32_t nf = P.nfree;
  const size_t m = 6 * size_t(std::max(nf, 1));
  cudaStream_t st = P.stream;
  float* d = P.d_mx;
  float* r32 = d + m;
  float* z32 = d + 2 * m;
  float* p32 = d + 3 * m;
  float* q32 = d + 4 * m;
  MixedScalars* s = static_cast<MixedScalars*>(P.d_ms);
  MixedScalars* hs = static_cast<MixedScalars*>(P.h_ms);
  SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
  SVXG_CUDA(cudaStreamSynchronize(st));
  const double bn = hs->bn;
  const double target = rtol * bn;
  if (!std::isfinite(bn) || !std::isfinite(hs->rn)) {
    out.rel_res = INFINITY;
    out.breakdown = 1;
    P.active = false;
    if (res) *res = out;
    return SVXG_OK;
  }
  out.rel_res = bn > 0 ? hs->rn / bn : 0.0;
  if (hs->rn <= target || !(bn > 0) || nf == 0 || (hs->done && hs->done != 3)) {
    out.converged = (hs->rn <= target || !(bn > 0) || nf == 0) ? 1 : 0;
    out.breakdown = hs->breakdown;
    if (res) *res = out;
    return SVXG_OK;
  }
  (k_resume<<<1, 32, 0, st>>>(s, target, maxit), SVXG_COUNT_LAUNCH());
  P.cycle_stop = &s->done;
  int32_t queued = 0, batch = 2;
  for (;;) {
    SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(cudaStreamSynchronize(st));
    if (hs->done || queued >= maxit) break;
    const int32_t todo = std::min(batch, maxit - queued);
    for (int32_t it = 0; it < todo; ++it) {
      (k_spmv32_dot<<<rblk(nf), kT, 0, st>>>(nf, P.K.rowptr, P.K.col, P.K.val32, p32, q32, P.d_partials,
                                             P.d_counter, s),
       SVXG_COUNT_LAUNCH());
      (k_axpy32<<<vblk(nf), kT, 0, st>>>(nf, d, r32, p32, q32, P.d_partials, P.d_counter, s), SVXG_COUNT_LAUNCH());
      (k_fold<<<vblk(nf), kT, 0, st>>>(nf, P.d_x, d, s, 0), SVXG_COUNT_LAUNCH());
      (k_spmv64_if<<<rblk(nf), kT, 0, st>>>(nf, P.K.rowptr, P.K.col, P.K.val, P.d_x, P.d_q, s, 0),
       SVXG_COUNT_LAUNCH());
      (k_true_resid<<<vblk(nf), kT, 0, st>>>(nf, P.d_f, P.d_q, r32, P.d_partials, P.d_counter, s, 0),
       SVXG_COUNT_LAUNCH());
      TRY(vcycle32(P, r32, z32));
      (k_rz32<1><<<vblk(nf), kT, 0, st>>>(nf, r32, z32, nullptr, P.d_partials, P.d_counter, s), SVXG_COUNT_LAUNCH());
      (k_p32<<<vblk(nf), kT, 0, st>>>(nf, z32, p32, s), SVXG_COUNT_LAUNCH());
      (k_cap32<<<1, 32, 0, st>>>(s), SVXG_COUNT_LAUNCH());
    }
    SVXG_CUDA(cudaGetLastError());
    queued += todo;
    batch = std::min(batch * 2, 32);
  }
  P.cycle_stop = nullptr;
  // the iterate is x + d: fold what is left (the next call's sequence is unchanged by it)
  (k_fold<<<vblk(nf), kT, 0, st>>>(nf, P.d_x, d, s, 1), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
  SVXG_CUDA(cudaStreamSynchronize(st));
  out.iters = hs->iters;
  out.converged = hs->converged;
  out.breakdown = hs->breakdown;
  out.rel_res = hs->converged ? hs->rel_res : (bn > 0 ? hs->rn / bn : 0.0);
  if (out.breakdown && !std::isfinite(hs->rn)) out.rel_res = INFINITY;
  P.run_iters += out.iters;
  if (res) *res = out;
  return SVXG_OK;
}

}  // namespace svxg
