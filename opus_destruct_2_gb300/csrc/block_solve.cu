// block_solve.cu - a whole AMG-preconditioned iterate() of a small problem in one block launch.
//
// A small problem's iteration is a few dozen tiny kernels (the CG steps and, per level, the
// smoothing, residual, restriction, prolongation and coarse-solve products); their launches, not
// their arithmetic, set its cost, and when many problems run at once the GPU's launch rate is the
// bound. Here one block of 1024 threads runs the iterations of pcg_iterate - the same steps, the
// same breakdown and stopping rules, the same device scalars (solve.cu's plain_body) - and inside
// each the same V-cycle as vcycle.cu (degree-2 Chebyshev in D^-1 A on [lmax/10, lmax] before and
// after the coarse correction, FP32, the coarsest level solved by its dense inverse), with block
// barriers in place of kernel boundaries. Products are one thread per (row, component) over the
// row's blocks; dot products are fixed-order block trees; the coarsest solve applies an FP32 copy
// of L^-1 (the cycle is FP32 throughout). Results are deterministic and tolerance-equal to the
// multi-kernel path, which larger problems keep.
#include <algorithm>
#include <cmath>

#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 1024;
constexpr int kMaxLevels = 16;

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

struct BLevel {
  int32_t n;
  const int32_t* rowptr;
  const int32_t* col;
  const float* val;   // A (f32)
  const float* dinv;  // D^-1 (f32)
  const int32_t* prow;
  const int32_t* pcol;
  const float* pval;  // P by fine row (to the next level)
  const int32_t* rrow;
  const int32_t* rent_i;
  const float* rval;  // P^T by coarse row
  float *b, *x, *r, *d0, *d1;
  float inv_theta, c1[8], c2[8];
  int32_t degree;     // smoothing degree (the stalled coarsest: its polynomial in place of a solve)
};

struct BDesc {
  int32_t levels, chol_n;
  const float* cinv;  // L^-1 then L^-T (f32, chol_n^2 each)
  BLevel lv[kMaxLevels];
};

__device__ __forceinline__ double tree_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int d = kT / 2; d > 0; d >>= 1) {
    if (int(threadIdx.x) < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  const double t = sh[0];
  __syncthreads();
  return t;
}

// (A v)_t for entry t = 6 i + c of a BSR operator (f32)
__device__ __forceinline__ float bsr_entry(int64_t t, const int32_t* rowptr, const int32_t* col, const float* val,
                                           const float* v) {
  const int32_t i = int32_t(t / 6);
  const int c = int(t % 6);
  float y = 0.0f;
  for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const float* a = val + 36 * int64_t(k) + 6 * c;
    const float* w = v + 6 * int64_t(col[k]);
    y += a[0] * w[0] + a[1] * w[1] + a[2] * w[2] + a[3] * w[3] + a[4] * w[4] + a[5] * w[5];
  }
  return y;
}

// out = D^-1 in (per node), times s
__device__ __forceinline__ void dinv_apply(int32_t n, const float* D, const float* in, float s, float* out) {
  for (int32_t i = threadIdx.x; i < n; i += kT) {
    const float* Di = D + 36 * int64_t(i);
    float v[6];
    for (int q = 0; q < 6; ++q) v[q] = in[6 * int64_t(i) + q];
    for (int c = 0; c < 6; ++c) {
      float a = 0.0f;
      for (int q = 0; q < 6; ++q) a += Di[6 * c + q] * v[q];
      out[6 * int64_t(i) + c] = a * s;
    }
  }
}

// Chebyshev smoothing of A x = b (vcycle.cu's smooth): from zero, or from x; leaves r = b - A x
__device__ void smooth(const BLevel& L, const float* b, float* x, bool from_zero) {
  const int64_t m = 6 * int64_t(L.n);
  float* d = L.d0;
  float* dn = L.d1;
  if (from_zero) {
    dinv_apply(L.n, L.dinv, b, L.inv_theta, d);
    __syncthreads();
    for (int64_t t = threadIdx.x; t < m; t += kT) x[t] = 0.0f;
  } else {
    for (int64_t t = threadIdx.x; t < m; t += kT) L.r[t] = b[t] - bsr_entry(t, L.rowptr, L.col, L.val, x);
    __syncthreads();
    dinv_apply(L.n, L.dinv, L.r, L.inv_theta, d);
  }
  __syncthreads();
  for (int i = 1; i < L.degree; ++i) {
    // x += d; r = b - A x; dn = c1 d + c2 D^-1 r
    for (int64_t t = threadIdx.x; t < m; t += kT) x[t] += d[t];
    __syncthreads();
    for (int64_t t = threadIdx.x; t < m; t += kT) L.r[t] = b[t] - bsr_entry(t, L.rowptr, L.col, L.val, x);
    __syncthreads();
    dinv_apply(L.n, L.dinv, L.r, L.c2[i], dn);
    __syncthreads();
    for (int64_t t = threadIdx.x; t < m; t += kT) dn[t] += L.c1[i] * d[t];
    __syncthreads();
    float* tmp = d;
    d = dn;
    dn = tmp;
  }
  for (int64_t t = threadIdx.x; t < m; t += kT) x[t] += d[t];
  __syncthreads();
  for (int64_t t = threadIdx.x; t < m; t += kT) L.r[t] = b[t] - bsr_entry(t, L.rowptr, L.col, L.val, x);
  __syncthreads();
}

// one V-cycle from zero on levels[0] for b = lv[0].b, result in lv[0].x
__device__ void vcycle_block(const BDesc& D) {
  const int last = D.levels - 1;
  for (int l = 0; l < last; ++l) {
    const BLevel& L = D.lv[l];
    const BLevel& C = D.lv[l + 1];
    smooth(L, L.b, L.x, true);
    // restriction: C.b = P^T r
    for (int64_t t = threadIdx.x; t < 6 * int64_t(C.n); t += kT)
      C.b[t] = bsr_entry(t, L.rrow, L.rent_i, L.rval, L.r);
    __syncthreads();
  }
  {
    const BLevel& L = D.lv[last];
    if (D.chol_n > 0) {
      const int32_t m = D.chol_n;
      // x = L^-T (L^-1 b): rows of L^-1, then rows of L^-T (f32), a warp per row
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      for (int32_t row = w; row < m; row += kT / 32) {
        const float* Mr = D.cinv + int64_t(row) * m;
        float s = 0.0f;
        for (int32_t k = lane; k < m; k += 32) s += Mr[k] * L.b[k];
        for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
        if (lane == 0) L.r[row] = s;
      }
      __syncthreads();
      for (int32_t row = w; row < m; row += kT / 32) {
        const float* Mr = D.cinv + int64_t(m) * m + int64_t(row) * m;
        float s = 0.0f;
        for (int32_t k = lane; k < m; k += 32) s += Mr[k] * L.r[k];
        for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
        if (lane == 0) L.x[row] = s;
      }
      __syncthreads();
    } else {
      smooth(L, L.b, L.x, true);
    }
  }
  for (int l = last - 1; l >= 0; --l) {
    const BLevel& L = D.lv[l];
    const BLevel& C = D.lv[l + 1];
    // prolongation: x += P xc
    for (int64_t t = threadIdx.x; t < 6 * int64_t(L.n); t += kT) L.x[t] += bsr_entry(t, L.prow, L.pcol, L.pval, C.x);
    __syncthreads();
    smooth(L, L.b, L.x, false);
  }
}

__global__ void __launch_bounds__(kT) k_amg_pcg_block(int32_t nf, const int32_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ col, const double* __restrict__ val,
                                                      const BDesc* __restrict__ desc, double* x, double* r, double* z,
                                                      double* p, double* q, PcgScalars* s) {
  __shared__ double sh[kT];
  const BDesc& D = *desc;
  const BLevel& L0 = D.lv[0];
  const int64_t m = 6 * int64_t(nf);
  for (int32_t guard = 0; guard <= s->maxit; ++guard) {
    __syncthreads();
    if (s->done) break;
    // q = K p (FP64), p.q, alpha
    double pq = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += kT) {
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
    pq = tree_sum(pq, sh);
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
    const double alpha = s->alpha;
    double rr = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += kT) {
      x[t] += alpha * p[t];
      const double rv = r[t] - alpha * q[t];
      r[t] = rv;
      rr += rv * rv;
      L0.b[t] = float(rv);
    }
    rr = tree_sum(rr, sh);
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
    // z = M^-1 r, r.z, beta
    vcycle_block(D);
    double rz = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += kT) {
      const double zv = double(L0.x[t]);
      z[t] = zv;
      rz += r[t] * zv;
    }
    rz = tree_sum(rz, sh);
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
    const double beta = s->beta;
    for (int64_t t = threadIdx.x; t < m; t += kT) p[t] = z[t] + beta * p[t];
    __syncthreads();
    if (threadIdx.x == 0 && !s->done && s->iters >= s->maxit) s->done = 2;
  }
}

__global__ void k_to_f32(int64_t n, const double* a, float* b) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) b[k] = float(a[k]);
}

void cheb_coeffs(double lmax, double ratio, int degree, BLevel* L) {
  const double lmin = lmax / ratio;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  L->inv_theta = float(1.0 / theta);
  L->degree = degree;
  for (int i = 1; i < degree && i < 8; ++i) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    L->c1[i] = float(rn * rho);
    L->c2[i] = float(2.0 * rn / delta);
    rho = rn;
  }
}

}  // namespace

bool block_solve_fits(const Problem& P) {
  return !P.jacobi_only && !P.lv.empty() && P.pc_n == P.nfree && P.nfree > 0 && P.nfree <= kBlockSolveMax &&
         int(P.lv.size()) <= kMaxLevels && !P.spmv_timer() && P.seg_n == 0;
}

// the descriptor (and the FP32 coarsest inverse) of an assembled problem, made once
static int block_prepare(Problem& P) {
  if (P.d_bdesc) return SVXG_OK;
  cudaStream_t st = P.stream;
  BDesc h{};
  h.levels = int32_t(P.lv.size());
  h.chol_n = P.chol_n;
  if (P.chol_n > 0) {
    float* c32 = nullptr;
    TRY(P.mem.alloc(&c32, 2 * size_t(P.chol_n) * size_t(P.chol_n)));
    const int64_t cnt = 2 * int64_t(P.chol_n) * P.chol_n;
    (k_to_f32<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, P.d_cinv, c32), SVXG_COUNT_LAUNCH());
    P.d_cinv32 = c32;
    h.cinv = c32;
  }
  for (size_t l = 0; l < P.lv.size(); ++l) {
    const Level& L = P.lv[l];
    BLevel& B = h.lv[l];
    B.n = L.A.n;
    B.rowptr = L.A.rowptr;
    B.col = L.A.col;
    B.val = L.A.val32;
    B.dinv = L.dinv32;
    B.prow = L.prow;
    B.pcol = L.pcol;
    B.pval = L.pval32;
    B.rrow = L.rrow;
    B.rent_i = L.rent_i;
    B.rval = L.pval32 ? L.pval32 + 36 * L.pnnz : nullptr;
    B.b = L.b32;
    B.x = L.x32;
    B.r = L.r32;
    B.d0 = L.t32;
    B.d1 = L.u32;
    const bool last = l + 1 == P.lv.size();
    if (last && P.chol_n == 0) cheb_coeffs(L.cheb_lmax, 30.0, 8, &B);
    else cheb_coeffs(L.cheb_lmax, 10.0, 2, &B);
  }
  BDesc* d = nullptr;
  TRY(P.mem.alloc(reinterpret_cast<char**>(&d), sizeof(BDesc)));
  SVXG_CUDA(cudaMemcpyAsync(d, &h, sizeof(BDesc), cudaMemcpyHostToDevice, st));
  SVXG_CUDA(host_wait(st));  // (h is on the stack)
  P.d_bdesc = d;
  return SVXG_OK;
}

// the iterations of pcg_iterate in one launch (after k_iter_start; P.d_s holds the run's scalars)
int block_iterate(Problem& P) {
  TRY(block_prepare(P));
  (k_amg_pcg_block<<<1, kT, 0, P.stream>>>(P.nfree, P.K.rowptr, P.K.col, P.K.val, static_cast<const BDesc*>(P.d_bdesc),
                                           P.d_x, P.d_r, P.d_z, P.d_p, P.d_q, P.d_s),
   SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

}  // namespace svxg
