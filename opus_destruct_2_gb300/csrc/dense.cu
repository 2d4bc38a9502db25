// dense.cu - the coarsest level's dense factor and its inverse, tiled over many SMs.
//
// Restates factor_coarsest (core/src/solve/amg.cpp:535-578): the coarsest operator (m x m, m =
// 6 n_c <= 1152) is symmetrized, factored as L L^T with the pivot floor max(1e-12 dmax, 1e-300),
// and the cycle's coarsest solve (amg.cpp:580-592) applies L^-T L^-1. Here the factor is a
// right-looking blocked Cholesky on 32 x 32 tiles (per step: the diagonal tile in one CTA, the
// panel and the trailing update one CTA per tile), and L^-1 is built by tile diagonals
// (X_ij = -L_ii^-1 sum_k L_ik X_kj, all tiles of one diagonal at once); the cycle then needs two
// dense products instead of two sequential substitutions. FP64 throughout. The matrix is padded
// to a multiple of 32 with identity rows, which leaves the factor of the m x m block unchanged.
#include <cmath>

#include "problem.cuh"

namespace svxg {
namespace {

constexpr int TB = 32;    // tile side
constexpr int kDT = 256;  // threads per tile CTA: row t / 8, columns 4 (t % 8) .. + 3

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
  for (int e = threadIdx.x; e < TB * TB; e += kDT) {
    const int r = e / TB, c = e % TB;
    S[r][c] = D[int64_t(ti * TB + r) * mp + tj * TB + c];
  }
}

__device__ __forceinline__ void store_tile(double* __restrict__ D, int32_t mp, int32_t ti, int32_t tj,
                                           double (*S)[TB + 1]) {
  for (int e = threadIdx.x; e < TB * TB; e += kDT) {
    const int r = e / TB, c = e % TB;
    D[int64_t(ti * TB + r) * mp + tj * TB + c] = S[r][c];
  }
}

// step k, diagonal tile: L_kk (into D) and L_kk^-1 (into W + k * TB * TB, row-major, zero above)
__global__ void __launch_bounds__(kDT) k_potrf(int32_t k, int32_t mp, double* D, double* W, const double* dmax_p) {
  __shared__ double A[TB][TB + 1], X[TB][TB + 1];
  load_tile(A, D, mp, k, k);
  __syncthreads();
  const double floor_v = fmax(1e-12 * *dmax_p, 1e-300);
  for (int j = 0; j < TB; ++j) {
    if (threadIdx.x == 0) {
      double d = A[j][j];
      for (int q = 0; q < j; ++q) d -= A[j][q] * A[j][q];
      if (!(d > 1e-12 * *dmax_p)) d = floor_v;
      A[j][j] = sqrt(d);
    }
    __syncthreads();
    const int i = j + 1 + int(threadIdx.x);
    if (i < TB) {
      double v = A[i][j];
      for (int q = 0; q < j; ++q) v -= A[i][q] * A[j][q];
      A[i][j] = v / A[j][j];
    }
    __syncthreads();
  }
  // zero above the diagonal, then the inverse column by column (forward substitution)
  for (int e = threadIdx.x; e < TB * TB; e += kDT) {
    const int r = e / TB, c = e % TB;
    if (c > r) A[r][c] = 0.0;
    X[r][c] = 0.0;
  }
  __syncthreads();
  if (threadIdx.x < TB) {
    const int c = threadIdx.x;
    X[c][c] = 1.0 / A[c][c];
    for (int i = c + 1; i < TB; ++i) {
      double s = 0.0;
      for (int q = c; q < i; ++q) s += A[i][q] * X[q][c];
      X[i][c] = -s / A[i][i];
    }
  }
  __syncthreads();
  store_tile(D, mp, k, k, A);
  double* Wk = W + int64_t(k) * TB * TB;
  for (int e = threadIdx.x; e < TB * TB; e += kDT) Wk[e] = X[e / TB][e % TB];
}

// step k, panel: L_ik = A_ik L_kk^-T for i = k + 1 + blockIdx.x
__global__ void __launch_bounds__(kDT) k_trsm(int32_t k, int32_t mp, double* D, const double* __restrict__ W) {
  __shared__ double A[TB][TB + 1], X[TB][TB + 1];
  const int32_t i = k + 1 + int32_t(blockIdx.x);
  load_tile(A, D, mp, i, k);
  const double* Wk = W + int64_t(k) * TB * TB;
  for (int e = threadIdx.x; e < TB * TB; e += kDT) X[e / TB][e % TB] = Wk[e];
  __syncthreads();
  const int r = threadIdx.x / 8, c0 = 4 * (threadIdx.x % 8);
  double out[4];
  for (int u = 0; u < 4; ++u) {
    double s = 0.0;
    for (int q = 0; q < TB; ++q) s += A[r][q] * X[c0 + u][q];
    out[u] = s;
  }
  for (int u = 0; u < 4; ++u) D[int64_t(i * TB + r) * mp + k * TB + c0 + u] = out[u];
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
  const int r = threadIdx.x / 8, c0 = 4 * (threadIdx.x % 8);
  for (int u = 0; u < 4; ++u) {
    double s = 0.0;
    for (int q = 0; q < TB; ++q) s += A[r][q] * B[c0 + u][q];
    D[int64_t(i * TB + r) * mp + j * TB + c0 + u] -= s;
  }
}

// X_jj = L_jj^-1 (all diagonal tiles)
__global__ void __launch_bounds__(kDT) k_inv_diag(int32_t mp, const double* __restrict__ W, double* X) {
  const int32_t j = blockIdx.x;
  const double* Wj = W + int64_t(j) * TB * TB;
  for (int e = threadIdx.x; e < TB * TB; e += kDT) X[int64_t(j * TB + e / TB) * mp + j * TB + e % TB] = Wj[e];
}

// diagonal d of X = L^-1: X_ij = -L_ii^-1 sum_{k=j}^{i-1} L_ik X_kj, i = j + d, j = blockIdx.x
__global__ void __launch_bounds__(kDT) k_inv_step(int32_t d, int32_t mp, const double* __restrict__ D,
                                                  const double* __restrict__ W, double* X) {
  __shared__ double A[TB][TB + 1], B[TB][TB + 1];
  const int32_t j = blockIdx.x, i = j + d;
  const int r = threadIdx.x / 8, c0 = 4 * (threadIdx.x % 8);
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int32_t k = j; k < i; ++k) {
    load_tile(A, D, mp, i, k);
    load_tile(B, X, mp, k, j);
    __syncthreads();
    for (int u = 0; u < 4; ++u)
      for (int q = 0; q < TB; ++q) s[u] += A[r][q] * B[q][c0 + u];
    __syncthreads();
  }
  // B = S, A = L_ii^-1; X_ij = -A B
  for (int u = 0; u < 4; ++u) B[r][c0 + u] = s[u];
  const double* Wi = W + int64_t(i) * TB * TB;
  for (int e = threadIdx.x; e < TB * TB; e += kDT) A[e / TB][e % TB] = Wi[e];
  __syncthreads();
  for (int u = 0; u < 4; ++u) {
    double v = 0.0;
    for (int q = 0; q < TB; ++q) v += A[r][q] * B[q][c0 + u];
    X[int64_t(i * TB + r) * mp + j * TB + c0 + u] = -v;
  }
}

// the m x m results: chol = L below and on the diagonal, L^T above; cinv = X, then X^T
__global__ void k_dense_unpad(int32_t m, int32_t mp, const double* __restrict__ D, const double* __restrict__ X,
                              double* chol, double* cinv) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(m) * m) return;
  const int32_t i = int32_t(t / m), j = int32_t(t % m);
  chol[t] = i >= j ? D[int64_t(i) * mp + j] : D[int64_t(j) * mp + i];
  const double x = i >= j ? X[int64_t(i) * mp + j] : 0.0;
  cinv[t] = x;
  cinv[int64_t(m) * m + int64_t(j) * m + i] = x;
}

}  // namespace

// C (m x m, row-major, the coarsest operator as filled) -> P.d_chol (L with L^T mirrored above) and
// P.d_cinv (L^-1, then L^-T) - both m x m, allocated by the caller
int dense_factor_inverse(Problem& P, int32_t m, const double* C, double* chol, double* cinv) {
  if (m <= 0) return SVXG_OK;
  cudaStream_t st = P.stream;
  const int32_t T = (m + TB - 1) / TB, mp = T * TB;
  double *D = nullptr, *X = nullptr, *W = nullptr, *dmax = nullptr;
  const size_t dd = size_t(mp) * size_t(mp);
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&D), dd * sizeof(double), st));
  int e = SVXG_OK;
  if (pool_malloc_async(reinterpret_cast<void**>(&X), dd * sizeof(double), st) != cudaSuccess ||
      pool_malloc_async(reinterpret_cast<void**>(&W), size_t(T) * TB * TB * sizeof(double), st) != cudaSuccess ||
      pool_malloc_async(reinterpret_cast<void**>(&dmax), sizeof(double), st) != cudaSuccess) {
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
    if (cudaMemsetAsync(X, 0, dd * sizeof(double), st) != cudaSuccess) e = SVXG_ERR_CUDA;
    (k_inv_diag<<<unsigned(T), kDT, 0, st>>>(mp, W, X), SVXG_COUNT_LAUNCH());
    for (int32_t d = 1; d < T; ++d) (k_inv_step<<<unsigned(T - d), kDT, 0, st>>>(d, mp, D, W, X), SVXG_COUNT_LAUNCH());
    (k_dense_unpad<<<gblk(int64_t(m) * m, 256), 256, 0, st>>>(m, mp, D, X, chol, cinv), SVXG_COUNT_LAUNCH());
    if (cudaGetLastError() != cudaSuccess) {
      set_error("coarsest factor: kernel launch failed");
      e = SVXG_ERR_CUDA;
    }
  }
  for (void* q : {static_cast<void*>(D), static_cast<void*>(X), static_cast<void*>(W), static_cast<void*>(dmax)})
    if (q) cudaFreeAsync(q, st);
  return e;
}

}  // namespace svxg
