// mixed.cu - the mixed-precision solve: FP32 K and FP32 V-cycle inside FP64 iterative refinement.
//
//   outer (FP64):  r = f - K x   (K in FP64, the exact residual), stop when ||r|| <= rtol ||f||
//   inner (FP32):  K32 d = r32 by AMG-preconditioned CG to ||r_in|| <= tol_in ||r32||, from d = 0
//                  (tol_in = max(1e-4, 0.3 rtol ||f|| / ||r||): as few outer steps as f32 allows):
//                  SpMV and the V-cycle in FP32 (K32 is K rounded to f32, the cycle's own level-0
//                  operator), dot products with exact products and double-float partial sums,
//                  returned in FP64 (FF below)
//   update (FP64): x += d
// FP64 (or its double-float equal in the dots) stays in the outer residual, the dots and the
// coarsest dense factor. The refinement converges to the FP64 solution (its residual is the FP64
// K's), so the result meets the same rtol as the plain FP64 solve; each inner iteration reads half
// the bytes of an FP64 one and issues FP32 arithmetic (GB300's FP64 rate is a small fraction of
// FP32).
// Restarting the inner sequence at each outer step costs iterations (its Krylov space is lost),
// but a single f32 sequence with reliable updates does not converge on slender structures:
// f32 Krylov vectors lose conjugacy when the condition number times 2^-24 approaches 1. Each
// inner sequence runs as one graph launch (graphs.cu).
#include <cmath>

#include "problem.cuh"
#include "spmv_row.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;
constexpr int kRows = kT / 32;
// An inner FP32 sequence runs at most kInnerCap iterations; a restart that fails to cut the FP64
// residual to kMinGain of the previous one hands the run to the FP64 sequence.
constexpr int32_t kInnerCap = 60;
constexpr double kMinGain = 0.1;
inline unsigned vblk(int32_t n) { return unsigned((std::max(n, 1) + kT - 1) / kT); }

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

struct MixedScalars {
  double rz, pq, alpha, beta, rn_in, target_in, rr;
  int32_t iters, done, breakdown, maxit;
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

// Double-float sums for the inner dots. A pair (hi, lo) of floats, read as hi + lo, carries about
// 48 significant bits, and the product of two floats is exact in it; summing in pairs issues FP32
// instructions, where an FP64 sum of the same terms issues FP64 ones, which GB300 runs at a small
// fraction of the FP32 rate (in the fused SpMV the FP64 reduction, not the memory, set the time).
// The methods are published ones:
//   a thread's terms:    Dot2 (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
//                        Comput. 26 (2005), Alg. 5.3): TwoProduct by FMA, TwoSum of the high parts,
//                        the rounding errors summed beside them;
//   combining partials:  the accurate double-word addition (Joldes, Muller and Popescu, "Tight and
//                        rigorous error bounds for basic building blocks of double-word arithmetic",
//                        ACM TOMS 44 (2017), Alg. 6), relative error below 3u^2.
// The explicitly rounded intrinsics are never contracted into FMAs, which the error-free
// transformations need. The sums are combined in a fixed order: results are the same bits on every
// run, and the total is returned as an FP64 value.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return FF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ FF fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// Dot2 step: acc.hi the running sum of the products' high parts, acc.lo the sum of the errors
__device__ __forceinline__ void dot2_add(FF& acc, float x, float y) {
  const float h = __fmul_rn(x, y);
  const float r = __fmaf_rn(x, y, -h);
  const FF t = two_sum(acc.hi, h);
  acc.hi = t.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t.lo, r));
}

// a Dot2 accumulator as a normalised double-float value
__device__ __forceinline__ FF dot2_value(FF acc) { return two_sum(acc.hi, acc.lo); }

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  FF s = two_sum(a.hi, b.hi);
  const FF t = two_sum(a.lo, b.lo);
  s = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

// lanes xor-combined from `first` down (16: the whole warp; 4: lanes 0-7)
__device__ __forceinline__ FF ff_warp_sum(FF v, int first) {
  for (int d = first; d > 0; d >>= 1)
    v = ff_add(v, FF{__shfl_xor_sync(0xffffffffu, v.hi, d), __shfl_xor_sync(0xffffffffu, v.lo, d)});
  return v;
}

// the block's sum in thread 0
__device__ __forceinline__ FF ff_block_sum(FF v, float2* sh, int first) {
  v = ff_warp_sum(v, first);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = make_float2(v.hi, v.lo);
  __syncthreads();
  FF s{0.0f, 0.0f};
  if (w == 0) {
    if (lane < int(blockDim.x) / 32) s = FF{sh[lane].x, sh[lane].y};
    s = ff_warp_sum(s, 16);
  }
  return s;
}

// last-block reduction of double-float partials (stored as float pairs in the FP64 partials
// buffer); true in every thread of the last block, the FP64 total in tot
__device__ __forceinline__ bool reduce_last_ff(FF v, int first, double* partials, unsigned* counter, double* tot) {
  __shared__ float2 sh[32];
  __shared__ bool last;
  float2* pp = reinterpret_cast<float2*>(partials);
  const FF bs = ff_block_sum(v, sh, first);
  if (threadIdx.x == 0) {
    pp[blockIdx.x] = make_float2(bs.hi, bs.lo);
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  FF s{0.0f, 0.0f};
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    const float2 x = __ldcg(&pp[b]);
    s = ff_add(s, FF{x.x, x.y});
  }
  const FF t = ff_block_sum(s, sh, 16);
  if (threadIdx.x == 0) {
    *tot = double(t.hi) + double(t.lo);
    *counter = 0u;
  }
  return true;
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

// y32 = K32 p32, p.y in double-float -> alpha. Each warp takes kDotSteps row steps (the block's
// warps on consecutive warp indices at every step), so the block reduction and the wait on the
// partials' fence and counter are paid once per kDotSteps steps (measured on the city block: 1 step
// 48 us, 2 steps 42, 4 steps 40, 8 steps 44, the last with a partial last wave).
constexpr int kDotSteps = 4;
template <int SCHED>
inline unsigned spmv_dot_blocks(int32_t n) {
  const int64_t per = int64_t(kRows) * kDotSteps * RowMap<SCHED>::kRowsPerWarp;
  return unsigned((std::max<int64_t>(n, 1) + per - 1) / per);
}

template <int SCHED>
__global__ void __launch_bounds__(kT) k_spmv32_dot(int32_t n, const int32_t* __restrict__ rowptr,
                                                   const int32_t* __restrict__ col, const float* __restrict__ val,
                                                   const float* __restrict__ p, float* __restrict__ q,
                                                   double* partials, unsigned* counter, MixedScalars* s) {
  if (s->done) return;
  FF acc{0.0f, 0.0f};
  for (int j = 0; j < kDotSteps; ++j) {
    int c;
    bool lane_ok;
    const int32_t warp = (int32_t(blockIdx.x) * kDotSteps + j) * kRows + (threadIdx.x >> 5);
    const int32_t row = sched_row_of<SCHED>(warp, &c, &lane_ok);
    const bool row_ok = row < n;
    if (SCHED == kWarpRow && !row_ok) break;  // (warp-uniform; the warp's rows only grow)
    const float y = sched_row_product<SCHED, float, float, float>(row_ok, row, rowptr, col, val, p);
    if (row_ok && lane_ok) {
      q[6 * int64_t(row) + c] = y;
      dot2_add(acc, p[6 * int64_t(row) + c], y);
    }
  }
  // kWarpRow: only lanes 0-5 hold terms
  double tot;
  if (reduce_last_ff(dot2_value(acc), SCHED == kWarpRow ? 4 : 16, partials, counter, &tot) && threadIdx.x == 0) {
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

// d += alpha p, r -= alpha q (f32), ||r|| -> inner convergence
__global__ void k_axpy32(int32_t nf, float* __restrict__ d, float* __restrict__ r, const float* __restrict__ p,
                         const float* __restrict__ q, double* partials, unsigned* counter, MixedScalars* s) {
  if (s->done) return;
  const float a = float(s->alpha);
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  FF rr{0.0f, 0.0f};
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const int64_t k = 6 * i + c;
      d[k] += a * p[k];
      const float rv = r[k] - a * q[k];
      r[k] = rv;
      dot2_add(rr, rv, rv);
    }
  double tot;
  if (reduce_last_ff(dot2_value(rr), 16, partials, counter, &tot) && threadIdx.x == 0) {
    s->rn_in = sqrt(tot);
    if (s->rn_in <= s->target_in) s->done = 1;
  }
}

// r.z (f64 accumulation); MODE 0: start (rz, p = z), 1: iteration (beta)
template <int MODE>
__global__ void k_rz32(int32_t nf, const float* __restrict__ r, const float* __restrict__ z, float* p, double* partials,
                       unsigned* counter, MixedScalars* s) {
  if (MODE == 1 && s->done) return;
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  FF rz{0.0f, 0.0f};
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const float zv = z[6 * i + c];
      dot2_add(rz, r[6 * i + c], zv);
      if (MODE == 0) p[6 * i + c] = zv;
    }
  double tot;
  if (reduce_last_ff(dot2_value(rz), 16, partials, counter, &tot) && threadIdx.x == 0) {
    if (MODE == 0) {
      s->rz = tot;
      if (!(tot > 0)) {
        s->breakdown = !(tot == 0.0);
        s->done = 1;
      }
    } else if (!(tot > 0)) {
      s->breakdown = 1;
      s->done = 1;
    } else {
      s->beta = tot / s->rz;
      s->rz = tot;
    }
    if (MODE == 1 && !s->done && s->iters >= s->maxit) s->done = 1;
  }
}

__global__ void k_p32(int32_t nf, const float* __restrict__ z, float* __restrict__ p, const MixedScalars* s) {
  if (s->done) return;
  const float b = float(s->beta);
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  if (i < nf)
    for (int c = 0; c < 6; ++c) p[6 * i + c] = z[6 * i + c] + b * p[6 * i + c];
}

// outer: r64 = f - q64 (q64 = K x), ||r||^2 -> rr; r32 = f32(r64); inner state reset
__global__ void k_outer_resid(int32_t nf, const double* __restrict__ f, const double* __restrict__ q,
                              double* __restrict__ r64, float* __restrict__ r32, float* __restrict__ d,
                              double* partials, unsigned* counter, MixedScalars* s, double tol_in, int32_t maxit) {
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  double rr = 0.0;
  if (i < nf)
    for (int c = 0; c < 6; ++c) {
      const int64_t k = 6 * i + c;
      const double rv = f[k] - q[k];
      r64[k] = rv;
      r32[k] = float(rv);
      d[k] = 0.0f;
      rr += rv * rv;
    }
  double tot;
  if (reduce_last(rr, partials, counter, &tot) && threadIdx.x == 0) {
    s->rr = tot;
    s->target_in = tol_in * sqrt(tot);
    s->done = 0;
    s->breakdown = 0;
    s->maxit = maxit;
  }
}

// x += d (f64 += f32)
__global__ void k_outer_update(int32_t nf, double* __restrict__ x, const float* __restrict__ d) {
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  if (i < nf)
    for (int c = 0; c < 6; ++c) x[6 * i + c] += double(d[6 * i + c]);
}

// one inner iteration, enqueued on P.stream
int mixed_body(Problem& P) {
  const int32_t nf = P.nfree;
  const size_t m = 6 * size_t(std::max(nf, 1));
  cudaStream_t st = P.stream;
  float* d = P.d_mx;
  float* r32 = d + m;
  float* z32 = d + 2 * m;
  float* p32 = d + 3 * m;
  float* q32 = d + 4 * m;
  MixedScalars* s = static_cast<MixedScalars*>(P.d_ms);
  if (P.spmv_timer()) TRY(timer_mark(P));
  if (P.sched_k32 == kGroupRow)
    (k_spmv32_dot<kGroupRow><<<spmv_dot_blocks<kGroupRow>(nf), kT, 0, st>>>(nf, P.K.rowptr, P.K.col, P.K.val32, p32,
                                                                          q32, P.d_partials, P.d_counter, s),
     SVXG_COUNT_LAUNCH());
  else
    (k_spmv32_dot<kWarpRow><<<spmv_dot_blocks<kWarpRow>(nf), kT, 0, st>>>(nf, P.K.rowptr, P.K.col, P.K.val32, p32,
                                                                        q32, P.d_partials, P.d_counter, s),
     SVXG_COUNT_LAUNCH());
  if (P.spmv_timer()) TRY(timer_mark(P, true));
  (k_axpy32<<<vblk(nf), kT, 0, st>>>(nf, d, r32, p32, q32, P.d_partials, P.d_counter, s), SVXG_COUNT_LAUNCH());
  TRY(vcycle32(P, r32, z32));
  (k_rz32<1><<<vblk(nf), kT, 0, st>>>(nf, r32, z32, nullptr, P.d_partials, P.d_counter, s), SVXG_COUNT_LAUNCH());
  (k_p32<<<vblk(nf), kT, 0, st>>>(nf, z32, p32, s), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

__global__ void k_fill_ones32(int32_t nf, float* x) {
  const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
  if (i < nf)
    for (int c = 0; c < 6; ++c) x[6 * i + c] = 1.0f;
}

}  // namespace

// The mixed sequence's SpMV timed alone (solve.cu's time_cg_spmv for K32): `reps` launches of
// k_spmv32_dot, each doing its work (scratch scalars with done = 0), p = 1.
int time_cg_spmv32(Problem& P, int32_t reps, float* ms_per_launch) {
  *ms_per_launch = 0.0f;
  if (P.nfree <= 0 || reps <= 0 || !P.K.val32 || !P.d_partials) return SVXG_OK;
  const int32_t nf = P.nfree;
  const size_t m = 6 * size_t(nf);
  float *x = nullptr, *y = nullptr;
  MixedScalars* s = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&x), m * sizeof(float), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&y), m * sizeof(float), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&s), sizeof(MixedScalars), P.stream));
  SVXG_CUDA(cudaMemsetAsync(s, 0, sizeof(MixedScalars), P.stream));
  (k_fill_ones32<<<vblk(nf), kT, 0, P.stream>>>(nf, x), SVXG_COUNT_LAUNCH());
  auto launch = [&] {
    if (P.sched_k32 == kGroupRow)
      (k_spmv32_dot<kGroupRow><<<spmv_dot_blocks<kGroupRow>(nf), kT, 0, P.stream>>>(nf, P.K.rowptr, P.K.col,
                                                                                    P.K.val32, x, y, P.d_partials,
                                                                                    P.d_counter, s),
       SVXG_COUNT_LAUNCH());
    else
      (k_spmv32_dot<kWarpRow><<<spmv_dot_blocks<kWarpRow>(nf), kT, 0, P.stream>>>(nf, P.K.rowptr, P.K.col, P.K.val32,
                                                                                  x, y, P.d_partials, P.d_counter, s),
       SVXG_COUNT_LAUNCH());
  };
  cudaEvent_t e0, e1;
  SVXG_CUDA(cudaEventCreate(&e0));
  SVXG_CUDA(cudaEventCreate(&e1));
  launch();  // (warm-up)
  SVXG_CUDA(cudaEventRecord(e0, P.stream));
  for (int32_t r = 0; r < reps; ++r) launch();
  SVXG_CUDA(cudaEventRecord(e1, P.stream));
  int32_t done_iters = -1;
  SVXG_CUDA(cudaMemcpyAsync(&done_iters, &s->iters, sizeof(int32_t), cudaMemcpyDeviceToHost, P.stream));
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
    set_error("time_cg_spmv32: " + std::to_string(done_iters) + " of " + std::to_string(reps + 1) + " launches ran");
    return SVXG_ERR_STATE;
  }
  *ms_per_launch = ms / float(reps);
  return SVXG_OK;
}

int mixed_begin(Problem&) { return SVXG_OK; }

// The mixed-precision run: x (FP64, free-DOF order, the warm start) and f are P's run vectors.
int mixed_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res) {
  svxg_pcg_result out{};
  const int32_t nf = P.nfree;
  cudaStream_t st = P.stream;
  const size_t m = 6 * size_t(std::max(nf, 1));
  if (!P.d_mx) {
    TRY(P.mem.alloc(&P.d_mx, 5 * m));  // d, r32, z32, p32, q32
    MixedScalars* ms = nullptr;
    TRY(P.mem.alloc(&ms, 1));
    P.d_ms = ms;
    SVXG_CUDA(cudaMallocHost(&P.h_ms, sizeof(MixedScalars)));
  }
  float* d = P.d_mx;
  float* r32 = d + m;
  float* z32 = d + 2 * m;
  float* p32 = d + 3 * m;
  MixedScalars* s = static_cast<MixedScalars*>(P.d_ms);
  MixedScalars* hs = static_cast<MixedScalars*>(P.h_ms);
  double bn = 0.0;
  {
    // ||f|| from the begin() scalars
    SVXG_CUDA(cudaMemcpyAsync(P.h_s, P.d_s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    bn = P.h_s->bn;
  }
  const double target = rtol * bn;
  int32_t used = 0;
  if (!std::isfinite(bn)) {
    out.rel_res = INFINITY;
    out.breakdown = 1;
    P.active = false;
    if (res) *res = out;
    return SVXG_OK;
  }
  double rn_prev = INFINITY;
  bool fallback = false;
  for (int outer = 0; outer < 64; ++outer) {
    // r = f - K x in FP64
    TRY(spmv(P, P.K, P.d_x, P.d_q));
    SVXG_CUDA(cudaMemsetAsync(s, 0, sizeof(MixedScalars), st));
    (k_outer_resid<<<vblk(nf), kT, 0, st>>>(nf, P.d_f, P.d_q, P.d_r, r32, d, P.d_partials, P.d_counter, s, 1.0,
                                            std::min(maxit - used, kInnerCap)),
     SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    const double rn = std::sqrt(hs->rr);
    // the inner target: as deep as f32 allows, no deeper than needed
    const double tol_in = std::max(1e-4, 0.3 * target / std::max(rn, 1e-300));
    SVXG_CUDA(cudaMemcpyAsync(&s->target_in, &(hs->target_in = tol_in * rn), sizeof(double), cudaMemcpyHostToDevice,
                              st));
    out.rel_res = bn > 0 ? rn / bn : 0.0;
    if (!std::isfinite(rn)) {
      out.rel_res = INFINITY;
      out.breakdown = 1;
      break;
    }
    if (rn <= target || !(bn > 0) || nf == 0) {
      out.converged = 1;
      break;
    }
    if (used >= maxit) break;
    if (rn > kMinGain * rn_prev) {
      // the FP32 inner sequence no longer gains a factor 1/kMinGain per restart (an operator too
      // ill-conditioned for FP32 vectors): finish with the FP64 sequence from this x
      fallback = true;
      break;
    }
    rn_prev = rn;
    // inner CG from d = 0: z = M^-1 r32 (the f32 V-cycle), p = z
    P.cycle_stop = &s->done;
    TRY(vcycle32(P, r32, z32));
    (k_rz32<0><<<vblk(nf), kT, 0, st>>>(nf, r32, z32, p32, P.d_partials, P.d_counter, s), SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    if (hs->done) {
      // (the inner start already broke down or met its target)
    } else if (loop_graph_worth(P, P.loop_mixed)) {
      int64_t per = 0;
      P.mx_maxit = std::min(maxit - used, kInnerCap);
      TRY(run_loop(P, P.loop_mixed, &s->done, mixed_body, &per));
      SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
      SVXG_CUDA(host_wait(st));
      add_launches(per * std::max<int64_t>(1, hs->iters));
    } else {
      P.host_loops += 1;
      const size_t timed0 = P.timer_used;
      int32_t queued = 0, batch = 2;
      for (;;) {
        SVXG_CUDA(cudaMemcpyAsync(hs, s, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
        SVXG_CUDA(host_wait(st));
        const int32_t cap = std::min(maxit - used, kInnerCap);
        if (hs->done || queued >= cap) break;
        const int32_t todo = std::min(batch, cap - queued);
        for (int32_t it = 0; it < todo; ++it) TRY(mixed_body(P));
        queued += todo;
        batch = std::min(batch * 2, 32);
      }
      // (the live timer keeps the SpMV launches that did work: the first `iters` of the sequence)
      if (P.spmv_timer()) P.timer_used = std::min(P.timer_used, timed0 + size_t(std::max(hs->iters, 0)));
    }
    used += hs->iters;
    (k_outer_update<<<vblk(nf), kT, 0, st>>>(nf, P.d_x, d), SVXG_COUNT_LAUNCH());
    if (hs->breakdown && hs->iters == 0) {
      out.breakdown = 1;
      break;
    }
  }
  P.cycle_stop = nullptr;
  if (fallback) {
    svxg_pcg_result f64{};
    TRY(pcg_restart_fp64(P));
    TRY(plain_iterate(P, maxit - used, rtol, &f64));
    f64.iters += used;
    P.run_iters += used;
    P.mixed_fallbacks += 1;
    if (res) *res = f64;
    return SVXG_OK;
  }
  out.iters = used;
  P.run_iters += used;
  if (res) *res = out;
  return SVXG_OK;
}

}  // namespace svxg
