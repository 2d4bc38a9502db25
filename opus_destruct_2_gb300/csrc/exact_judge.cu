// exact_judge.cu - bond loads, utilizations and the failure set on the device (one thread per
// bond; compiled with -fmad=false so each bond's numbers are the reference's for the same u).
//
// Restates StressProblem::bond_load (core/src/stress/stress.cpp:477-502), bond_strength and
// bond_utilization (stress.cpp:14-57). The failure set {b : phi_b >= 1} comes back as bond
// indices in ascending order (flags, a scan, a scatter: no ordering by atomics).
#include "blk6.cuh"
#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;

__global__ void k_judge(int32_t nb, const svxg_bond* __restrict__ bonds, const svxg_node* __restrict__ nodes,
                        const svxg_material* __restrict__ mats, const double* __restrict__ u, double fragility,
                        svxg_bond_load* loads, double* phi, uint8_t* mode, int32_t* over_flag) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const svxg_bond b = bonds[k];
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
  if (loads) loads[k] = L;
  if (phi || mode || over_flag) {
    uint8_t m = 0;
    const double ph = bond_utilization(b, L, fragility, mats, &m);
    if (phi) phi[k] = ph;
    if (mode) mode[k] = m;
    if (over_flag) over_flag[k] = ph >= 1.0 ? 1 : 0;
  }
}

__global__ void k_compact(int32_t nb, const int32_t* flag, const int32_t* pos, int32_t* out) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nb && flag[k]) out[pos[k]] = k;
}

}  // namespace

int bond_loads_device(Problem& P, const double* u_nodes, svxg_bond_load* out) {
  if (P.nb == 0) return SVXG_OK;
  (k_judge<<<unsigned((P.nb + kT - 1) / kT), kT, 0, P.stream>>>(P.nb, P.d_bonds, P.d_nodes, P.d_mats, u_nodes, 1.0, out,
                                                              nullptr, nullptr, nullptr), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// phi, mode: device arrays (either may be null); over: device array of nb entries receiving the
// failing bonds in ascending order; *n_over: host.
int utilization_device(Problem& P, const double* u_nodes, double fragility, double* phi, uint8_t* mode,
                       int32_t* over, int32_t* n_over) {
  if (P.nb == 0) {
    if (n_over) *n_over = 0;
    return SVXG_OK;
  }
  int32_t *flag = nullptr, *pos = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&flag), sizeof(int32_t) * size_t(P.nb), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&pos), sizeof(int32_t) * size_t(P.nb), P.stream));
  const unsigned g = unsigned((P.nb + kT - 1) / kT);
  (k_judge<<<g, kT, 0, P.stream>>>(P.nb, P.d_bonds, P.d_nodes, P.d_mats, u_nodes, fragility, nullptr, phi, mode, flag), SVXG_COUNT_LAUNCH());
  int32_t total = 0;
  int e = exclusive_scan_i32(P, flag, pos, P.nb, &total);
  if (!e && over) (k_compact<<<g, kT, 0, P.stream>>>(P.nb, flag, pos, over), SVXG_COUNT_LAUNCH());
  cudaFreeAsync(flag, P.stream);
  cudaFreeAsync(pos, P.stream);
  if (e) return e;
  SVXG_CUDA(cudaGetLastError());
  if (n_over) *n_over = total;
  return SVXG_OK;
}

}  // namespace svxg
