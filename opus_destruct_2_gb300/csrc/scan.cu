// scan.cu - exclusive prefix sum of int32 arrays (reduce, scan the block sums, scan with offsets).
#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int32_t warp_incl(int32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ int32_t block_excl(int32_t v, int32_t* total) {
  __shared__ int32_t ws[kScanThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t inc = warp_incl(v);
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (w == 0) {
    int32_t s = lane < kScanThreads / 32 ? ws[lane] : 0;
    s = warp_incl(s);
    if (lane < kScanThreads / 32) ws[lane] = s;
  }
  __syncthreads();
  const int32_t before = (w > 0 ? ws[w - 1] : 0) + inc - v;
  *total = ws[kScanThreads / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void k_tile_sums(const int32_t* in, int64_t n, int32_t* sums) {
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  int32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + int64_t(k) * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  int32_t total;
  block_excl(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place, grand total to sums[ntiles]
__global__ void k_scan_sums(int32_t* sums, int64_t ntiles) {
  int32_t carry = 0;
  for (int64_t b0 = 0; b0 < ntiles; b0 += kScanThreads) {
    const int64_t i = b0 + threadIdx.x;
    const int32_t v = i < ntiles ? sums[i] : 0;
    int32_t total;
    const int32_t ex = block_excl(v, &total);
    if (i < ntiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) sums[ntiles] = carry;
}

__global__ void k_tile_scan(const int32_t* in, int32_t* out, int64_t n, const int32_t* sums) {
  // each thread owns kScanItems consecutive items
  const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int32_t total;
  int32_t run = block_excl(s, &total) + sums[blockIdx.x];
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

// one block for short arrays (at most one tile): out and the total (sums[0]) in one launch
__global__ void k_scan_one_tile(const int32_t* in, int32_t* out, int64_t n, int32_t* sums) {
  const int64_t base = int64_t(threadIdx.x) * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int32_t total;
  int32_t run = block_excl(s, &total);
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) sums[1] = total;
}

}  // namespace

int exclusive_scan_i32(Problem& P, const int32_t* in, int32_t* out, int64_t n, int32_t* total_host) {
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (P.scan_cap < ntiles + 1) {
    P.mem.release(P.d_scan);
    if (int e = P.mem.alloc(&P.d_scan, size_t(ntiles + 1))) return e;
    P.scan_cap = ntiles + 1;
  }
  if (n > 0 && ntiles == 1) {
    (k_scan_one_tile<<<1, kScanThreads, 0, P.stream>>>(in, out, n, P.d_scan), SVXG_COUNT_LAUNCH());
  } else if (n > 0) {
    (k_tile_sums<<<unsigned(ntiles), kScanThreads, 0, P.stream>>>(in, n, P.d_scan), SVXG_COUNT_LAUNCH());
    (k_scan_sums<<<1, kScanThreads, 0, P.stream>>>(P.d_scan, ntiles), SVXG_COUNT_LAUNCH());
    (k_tile_scan<<<unsigned(ntiles), kScanThreads, 0, P.stream>>>(in, out, n, P.d_scan), SVXG_COUNT_LAUNCH());
  } else {
    SVXG_CUDA(cudaMemsetAsync(P.d_scan, 0, sizeof(int32_t), P.stream));
  }
  SVXG_CUDA(cudaGetLastError());
  if (total_host) {
    SVXG_CUDA(cudaMemcpyAsync(total_host, P.d_scan + ntiles, sizeof(int32_t), cudaMemcpyDeviceToHost, P.stream));
    SVXG_CUDA(host_wait(P.stream));
  }
  return SVXG_OK;
}

const int32_t* scan_total_device(const Problem& P, int64_t n) {
  return P.d_scan + (n + kScanTile - 1) / kScanTile;
}

}  // namespace svxg
