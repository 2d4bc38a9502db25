// dense.cu - the coarsest level's dense factor and its inverse, spread over many SMs.
//
// Restates factor_coarsest (core/src/solve/amg.cpp:535-578): the coarsest operator (m x m, m =
// 6 n_c <= 1152) is symmetrized, factored as L L^T with the pivot floor max(1e-12 dmax, 1e-300),
// and the cycle's coarsest solve (amg.cpp:580-592) applies L^-T L^-1. The factor is a right-looking
// blocked Cholesky on 16 x 16 tiles (per step: the diagonal tile in one CTA, the panel and the
// trailing update one CTA per tile - small tiles, because an SM retires about one FP64 operation
// a cycle, so a tile's product is the step's critical path); L^-1 is then formed column by column,
// one warp per column (forward substitution on the identity, each step's dot product across the
// lanes), all columns at once. The cycle applies two dense products instead of two sequential
// substitutions. FP64 throughout. The matrix is padded to a multiple of 16 with identity rows,
// which leaves the factor of the m x m block unchanged.
#include <cmath>

#include "problem.cuh"

namespace svxg {
namespace {

constexpr int TB = 16;    // tile side
constexpr int kDT = 256;  // threads per tile CTA: entry (t / 16, t % 16)
constexpr int kMaxM = 1152;
constexpr int kInvWarps = 4;

inline unsigned gblk(int64_t n, int t) { return unsigned((std::max<int64_t>(n, 1) + t - 1) / t); }

// D (mp x mp, lower used) = the symmetrized matrix, identity on the padding
__global__ void k_dense_pad(int32_t m, int32_t mp, const double* __restrict__ C, double* __restrict__ D) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(mp) * mp) return;
  const int32_t i = int32_t(t / mp), j = int32_t(t % mp);
  double v = 0.0;
  if (i < m && j < m) {
    if (i > j) v = 0.5 * (C[int64_t(i) * m + j] + C[int64_t(j) * m + i]);
    else if (i == j) v = C[int64_t(i) * m + i];
  } else if (i == j) {
    v = 1.0;
  }
  D[t] = v;
}

__global__ void k_dense_dmax(int32_t m, const double* __restrict__ C, double* dmax) {
  __shared__ double sh[kDT];
  double d = 0.0;
  for (int32_t i = threadIdx.x; i < m; i += kDT) d = fmax(d, fabs(C[int64_t(i) * m + i]));
  sh[threadIdx.x] = d;
  __syncthreads();
  for (int s = kDT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *dmax = sh[0];
}

__device__ __forceinline__ void load_tile(double (*S)[TB + 1], const double* __restrict__ D, int32_t mp, int32_t ti,
                                          int32_t tj) {
  const int r = threadIdx.x / TB, c = threadIdx.x % TB;
  S[r][c] = D[int64_t(ti * TB + r) * mp + tj * TB + c];
}

// step k, diagonal tile: L_kk (into D) and L_kk^-1 (into W + k * TB * TB, row-major, zero above)
__global__ void __launch_bounds__(kDT) k_potrf(int32_t k, int32_t mp, double* D, double* W, const double* dmax_p) {
  __shared__ double A[TB][TB + 1], X[TB][TB + 1];
  __shared__ double rdiag[TB];  // 1 / L_jj (one division a column; an FP64 division is many operations)
  load_tile(A, D, mp, k, k);
  __syncthreads();
  const double dm = *dmax_p;
  for (int j = 0; j < TB; ++j) {
    if (threadIdx.x == 0) {
      double d = A[j][j];
      for (int q = 0; q < j; ++q) d -= A[j][q] * A[j][q];
      if (!(d > 1e-12 * dm)) d = fmax(1e-12 * dm, 1e-300);
      A[j][j] = sqrt(d);
      rdiag[j] = 1.0 / A[j][j];
    }
    __syncthreads();
    const int i = j + 1 + int(threadIdx.x);
    if (i < TB) {
      double v = A[i][j];
      for (int q = 0; q < j; ++q) v -= A[i][q] * A[j][q];
      A[i][j] = v * rdiag[j];
    }
    __syncthreads();
  }
  {
    const int r = threadIdx.x / TB, c = threadIdx.x % TB;
    if (c > r) A[r][c] = 0.0;
    X[r][c] = r == c ? rdiag[r] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < TB) {
    const int c = threadIdx.x;
    for (int i = c + 1; i < TB; ++i) {
      double s = 0.0;
      for (int q = c; q < i; ++q) s += A[i][q] * X[q][c];
      X[i][c] = -s * rdiag[i];
    }
  }
  __syncthreads();
  const int r = threadIdx.x / TB, c = threadIdx.x % TB;
  D[int64_t(k * TB + r) * mp + k * TB + c] = A[r][c];
  W[int64_t(k) * TB * TB + threadIdx.x] = X[r][c];
}

// step k, panel: L_ik = A_ik L_kk^-T for i = k + 1 + blockIdx.x
__global__ void __launch_bounds__(kDT) k_trsm(int32_t k, int32_t mp, double* D, const double* __restrict__ W) {
  __shared__ double A[TB][TB + 1], X[TB][TB + 1];
  const int32_t i = k + 1 + int32_t(blockIdx.x);
  load_tile(A, D, mp, i, k);
  const int r = threadIdx.x / TB, c = threadIdx.x % TB;
  X[r][c] = W[int64_t(k) * TB * TB + threadIdx.x];
  __syncthreads();
  double s = 0.0;
  for (int q = 0; q < TB; ++q) s += A[r][q] * X[c][q];
  D[int64_t(i * TB + r) * mp + k * TB + c] = s;
}

// step k, trailing update: D_ij -= L_ik L_jk^T over the tiles k < j <= i (one CTA each)
__global__ void __launch_bounds__(kDT) k_syrk(int32_t k, int32_t mp, double* D) {
  __shared__ double A[TB][TB + 1], B[TB][TB + 1];
  const int64_t idx = blockIdx.x;
  int32_t ii = int32_t((sqrt(8.0 * double(idx) + 1.0) - 1.0) * 0.5);
  while (int64_t(ii + 1) * (ii + 2) / 2 <= idx) ++ii;
  while (int64_t(ii) * (ii + 1) / 2 > idx) --ii;
  const int32_t jj = int32_t(idx - int64_t(ii) * (ii + 1) / 2);
  const int32_t i = k + 1 + ii, j = k + 1 + jj;
  load_tile(A, D, mp, i, k);
  load_tile(B, D, mp, j, k);
  __syncthreads();
  const int r = threadIdx.x / TB, c = threadIdx.x % TB;
  double s = 0.0;
  for (int q = 0; q < TB; ++q) s += A[r][q] * B[c][q];
  D[int64_t(i * TB + r) * mp + j * TB + c] -= s;
}

// rd = 1 / L_ii
__global__ void k_rdiag(int32_t m, int32_t mp, const double* __restrict__ D, double* rd) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) rd[i] = 1.0 / D[int64_t(i) * mp + i];
}

// L^-1 column j (one warp): x_j = 1 / L_jj, x_i = -(sum_{j<=q<i} L_iq x_q) / L_ii; written to
// cinv (L^-1, row-major m x m) and its transpose after it

__global__ void __launch_bounds__(32 * kInvWarps) k_inv_cols(int32_t m, int32_t mp, const double* __restrict__ D,
                                                             const double* __restrict__ rd, double* cinv) {
  __shared__ double x_sh[kInvWarps][kMaxM];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t j = int32_t(blockIdx.x) * kInvWarps + w;
  if (j >= m) return;
  double* x = x_sh[w];
  double* X = cinv;
  double* XT = cinv + int64_t(m) * m;
  for (int32_t i = lane; i < j; i += 32) {
    X[int64_t(i) * m + j] = 0.0;
    XT[int64_t(j) * m + i] = 0.0;
  }
  if (lane == 0) x[j] = rd[j];
  __syncwarp();
  for (int32_t i = j + 1; i < m; ++i) {
    const double* Li = D + int64_t(i) * mp;
    double s = 0.0;
    for (int32_t q = j + lane; q < i; q += 32) s += Li[q] * x[q];
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if (lane == 0) x[i] = -s * rd[i];
    __syncwarp();
  }
  for (int32_t i = j + lane; i < m; i += 32) {
    X[int64_t(i) * m + j] = x[i];
    XT[int64_t(j) * m + i] = x[i];
  }
}

// chol = L below and on the diagonal, L^T above (m x m)
__global__ void k_dense_unpad(int32_t m, int32_t mp, const double* __restrict__ D, double* chol) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(m) * m) return;
  const int32_t i = int32_t(t / m), j = int32_t(t % m);
  chol[t] = i >= j ? D[int64_t(i) * mp + j] : D[int64_t(j) * mp + i];
}

}  // namespace

// C (m x m, row-major, the coarsest operator as filled) -> chol (L with L^T mirrored above) and
// cinv (L^-1, then L^-T) - both m x m, allocated by the caller; chol may alias C
int dense_factor_inverse(Problem& P, int32_t m, const double* C, double* chol, double* cinv) {
  if (m <= 0) return SVXG_OK;
  if (m > kMaxM) {
    set_error("coarsest factor: more than 1152 unknowns");
    return SVXG_ERR_ARG;
  }
  cudaStream_t st = P.stream;
  const int32_t T = (m + TB - 1) / TB, mp = T * TB;
  double *D = nullptr, *W = nullptr, *dmax = nullptr, *rd = nullptr;
  const size_t dd = size_t(mp) * size_t(mp);
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&D), dd * sizeof(double), st));
  int e = SVXG_OK;
  if (pool_malloc_async(reinterpret_cast<void**>(&W), size_t(T) * TB * TB * sizeof(double), st) != cudaSuccess ||
      pool_malloc_async(reinterpret_cast<void**>(&dmax), sizeof(double), st) != cudaSuccess ||
      pool_malloc_async(reinterpret_cast<void**>(&rd), size_t(m) * sizeof(double), st) != cudaSuccess) {
    cudaGetLastError();
    set_error("coarsest factor: device allocation failed");
    e = SVXG_ERR_NOMEM;
  }
  if (!e) {
    (k_dense_dmax<<<1, kDT, 0, st>>>(m, C, dmax), SVXG_COUNT_LAUNCH());
    (k_dense_pad<<<gblk(int64_t(mp) * mp, 256), 256, 0, st>>>(m, mp, C, D), SVXG_COUNT_LAUNCH());
    for (int32_t k = 0; k < T; ++k) {
      (k_potrf<<<1, kDT, 0, st>>>(k, mp, D, W, dmax), SVXG_COUNT_LAUNCH());
      const int32_t rest = T - k - 1;
      if (rest > 0) {
        (k_trsm<<<unsigned(rest), kDT, 0, st>>>(k, mp, D, W), SVXG_COUNT_LAUNCH());
        (k_syrk<<<unsigned(int64_t(rest) * (rest + 1) / 2), kDT, 0, st>>>(k, mp, D), SVXG_COUNT_LAUNCH());
      }
    }
    (k_rdiag<<<gblk(m, 256), 256, 0, st>>>(m, mp, D, rd), SVXG_COUNT_LAUNCH());
    (k_inv_cols<<<unsigned((m + kInvWarps - 1) / kInvWarps), 32 * kInvWarps, 0, st>>>(m, mp, D, rd, cinv),
     SVXG_COUNT_LAUNCH());
    (k_dense_unpad<<<gblk(int64_t(m) * m, 256), 256, 0, st>>>(m, mp, D, chol), SVXG_COUNT_LAUNCH());
    if (cudaGetLastError() != cudaSuccess) {
      set_error("coarsest factor: kernel launch failed");
      e = SVXG_ERR_CUDA;
    }
  }
  for (void* q : {static_cast<void*>(D), static_cast<void*>(W), static_cast<void*>(dmax), static_cast<void*>(rd)})
    if (q) cudaFreeAsync(q, st);
  return e;
}

}  // namespace svxg
