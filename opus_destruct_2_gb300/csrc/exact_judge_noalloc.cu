// exact_judge_noalloc.cu - bond utilizations and the failure set with no device allocation.
//
// For hosts that own every byte of device memory themselves: an engine that reserves its HBM up
// front and hands out slices from its own pool, whose frame loop must neither block on
// cudaMalloc/cudaFree (both can synchronize the device) nor let a library grow the footprint
// outside the pool's accounting. Such a host cannot create a problem handle (that allocates), but
// it can keep the graph, the material table and a displacement in its own buffers and ask for the
// judge: phi, the failure mode and the ascending list of failing bonds, written into its own
// output buffers.
//
// The failure list needs scratch (a count and an offset per block of bonds); here it lives in one
// file-scope device array, so every GPU that loads this library holds it (512 KiB) until the
// process exits, and the largest graph is kMaxBonds bonds. Every call shares that array and leaves
// its contents behind: calls whose kernels overlap on the GPU (two host threads, or two streams,
// at once) race on it and must be ordered by the caller. Each call clears the two words that must
// start at zero (the invalid-input flag and the count) before its first kernel; the per-block
// entries are written before they are read in the same call.
//
// The per-bond numbers are the same device code as the problem's own judge (this file is compiled
// without FMA contraction, like it), so phi, mode and the list match it bit for bit.
#include <mutex>

#include "blk6.cuh"
#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;                   // bonds per block
constexpr int kMaxBlocks = 65536;         // -> at most kT * kMaxBlocks bonds
constexpr int64_t kMaxBonds = int64_t(kT) * kMaxBlocks;
constexpr int kScanT = 1024;
constexpr int kMaxDevices = 64;

// [0] invalid-input flag, [1] failing-bond count, [2, 2 + kMaxBlocks) per-block counts,
// [2 + kMaxBlocks, 2 + 2 kMaxBlocks) per-block offsets. In host code this name only stands for
// the array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) int32_t g_judge_scratch[2 + 2 * kMaxBlocks];

std::mutex g_setup_mu;
int32_t* g_scratch_ptr[kMaxDevices] = {};

// The scratch's device address on the current device, looked up on this device's first call.
int scratch_for_current_device(int32_t** out) {
  int dev = -1;
  SVXG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("svxg_utilization_noalloc: device ordinal beyond " + std::to_string(kMaxDevices));
    return SVXG_ERR_NODEVICE;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_judge_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("svxg_utilization_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return SVXG_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_scratch_ptr[dev];
  return SVXG_OK;
}

// phi of bond k (the problem's judge, restated over caller-owned arrays); false: bad indices
__device__ __forceinline__ bool judge_bond(int32_t k, int32_t n, const svxg_bond* __restrict__ bonds,
                                           const svxg_node* __restrict__ nodes, const svxg_material* __restrict__ mats,
                                           const double* __restrict__ u, double fragility, double* ph, uint8_t* md) {
  const svxg_bond b = bonds[k];
  if (b.a < 0 || b.a >= n || b.b >= n || b.ma >= SVXG_MAX_MATERIALS || b.mb >= SVXG_MAX_MATERIALS) return false;
  const svxg_node& na = nodes[b.a];
  const double* ua = na.fixed ? nullptr : u + 6 * int64_t(b.a);
  V3d cb = {0, 0, 0};
  const double* ub = nullptr;
  if (b.b >= 0) {
    const svxg_node& nbn = nodes[b.b];
    cb = v3of(nbn.c);
    ub = nbn.fixed ? nullptr : u + 6 * int64_t(b.b);
  }
  const svxg_bond_load L = bond_load(b, mats, v3of(na.c), ua, cb, ub);
  *ph = bond_utilization(b, L, fragility, mats, md);
  return true;
}

// phi and mode per bond; the block's failing-bond count into scratch[2 + block]
__global__ void __launch_bounds__(kT) k_na_judge(int32_t nb, int32_t n, const svxg_bond* __restrict__ bonds,
                                                 const svxg_node* __restrict__ nodes,
                                                 const svxg_material* __restrict__ mats, const double* __restrict__ u,
                                                 double fragility, double* phi, uint8_t* mode, int32_t* scratch) {
  const int32_t k = int32_t(blockIdx.x) * kT + int32_t(threadIdx.x);
  int over = 0;
  if (k < nb) {
    double ph = 0.0;
    uint8_t m = 0;
    if (judge_bond(k, n, bonds, nodes, mats, u, fragility, &ph, &m)) {
      if (phi) phi[k] = ph;
      if (mode) mode[k] = m;
      over = ph >= 1.0 ? 1 : 0;
    } else {
      atomicOr(scratch, 1);
    }
  }
  const int cnt = __syncthreads_count(over);
  if (threadIdx.x == 0) scratch[2 + blockIdx.x] = cnt;
}

// exclusive scan of the nblk block counts (one block), the total into scratch[1]
__global__ void __launch_bounds__(kScanT) k_na_scan(int32_t nblk, int32_t* scratch) {
  __shared__ int32_t warp_sum[kScanT / 32];
  const int32_t* cnt = scratch + 2;
  int32_t* off = scratch + 2 + kMaxBlocks;
  const int32_t per = (nblk + kScanT - 1) / kScanT;
  const int32_t i0 = int32_t(threadIdx.x) * per, i1 = min(nblk, i0 + per);
  int32_t s = 0;
  for (int32_t i = i0; i < i1; ++i) s += cnt[i];
  // inclusive scan of the threads' sums: within warps, then over the warps' totals
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t v = s;
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += t;
  }
  if (lane == 31) warp_sum[w] = v;
  __syncthreads();
  if (w == 0) {
    int32_t x = warp_sum[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += t;
    }
    warp_sum[lane] = x;
  }
  __syncthreads();
  int32_t run = v - s + (w > 0 ? warp_sum[w - 1] : 0);
  for (int32_t i = i0; i < i1; ++i) {
    off[i] = run;
    run += cnt[i];
  }
  if (threadIdx.x == kScanT - 1) scratch[1] = run;
}

// the failing bonds in ascending order: block offset + rank of the bond among its block's failures
__global__ void __launch_bounds__(kT) k_na_list(int32_t nb, int32_t n, const svxg_bond* __restrict__ bonds,
                                                const svxg_node* __restrict__ nodes,
                                                const svxg_material* __restrict__ mats, const double* __restrict__ u,
                                                double fragility, const int32_t* scratch, int32_t* over) {
  __shared__ int32_t warp_cnt[kT / 32];
  const int32_t k = int32_t(blockIdx.x) * kT + int32_t(threadIdx.x);
  bool f = false;
  if (k < nb) {
    double ph = 0.0;
    uint8_t m = 0;
    f = judge_bond(k, n, bonds, nodes, mats, u, fragility, &ph, &m) && ph >= 1.0;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, f);
  if (lane == 0) warp_cnt[w] = __popc(bal);
  __syncthreads();
  if (f) {
    int32_t r = scratch[2 + kMaxBlocks + blockIdx.x] + __popc(bal & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) r += warp_cnt[i];
    over[r] = k;
  }
}

}  // namespace
}  // namespace svxg

using namespace svxg;

extern "C" int svxg_utilization_noalloc(const svxg_node* nodes_dev, int32_t n, const svxg_bond* bonds_dev, int32_t nb,
                                        const svxg_material* mats_dev, const double* u_dev, double fragility,
                                        double* phi_dev, uint8_t* mode_dev, int32_t* over_dev, int32_t* n_over,
                                        void* stream) {
  if (n < 0 || nb < 0) {
    set_error("svxg_utilization_noalloc: negative size");
    return SVXG_ERR_ARG;
  }
  if (int64_t(nb) > kMaxBonds) {
    set_error("svxg_utilization_noalloc: " + std::to_string(nb) + " bonds exceed the maximum of " +
              std::to_string(kMaxBonds) + " (use svxg_utilization_device)");
    return SVXG_ERR_ARG;
  }
  if (nb == 0) {
    if (n_over) *n_over = 0;
    return SVXG_OK;
  }
  if (!nodes_dev || !bonds_dev || !mats_dev || !u_dev || n == 0) {
    set_error("svxg_utilization_noalloc: null graph array or no nodes");
    return SVXG_ERR_ARG;
  }
  int32_t* scratch = nullptr;
  const int e = scratch_for_current_device(&scratch);
  if (e) return e;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int32_t nblk = int32_t((int64_t(nb) + kT - 1) / kT);
  SVXG_CUDA(cudaMemsetAsync(scratch, 0, 2 * sizeof(int32_t), st));
  (k_na_judge<<<unsigned(nblk), kT, 0, st>>>(nb, n, bonds_dev, nodes_dev, mats_dev, u_dev, fragility, phi_dev, mode_dev,
                                              scratch), SVXG_COUNT_LAUNCH());
  (k_na_scan<<<1, kScanT, 0, st>>>(nblk, scratch), SVXG_COUNT_LAUNCH());
  if (over_dev)
    (k_na_list<<<unsigned(nblk), kT, 0, st>>>(nb, n, bonds_dev, nodes_dev, mats_dev, u_dev, fragility, scratch,
                                               over_dev), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  int32_t head[2] = {0, 0};
  SVXG_CUDA(cudaMemcpyAsync(head, scratch, sizeof(head), cudaMemcpyDeviceToHost, st));
  SVXG_CUDA(cudaStreamSynchronize(st));
  if (head[0]) {
    set_error("svxg_utilization_noalloc: a bond's node index or material id is out of range");
    return SVXG_ERR_ARG;
  }
  if (n_over) *n_over = head[1];
  return SVXG_OK;
}
