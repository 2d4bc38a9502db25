// exact_cascade.cu - the device side of the judge's break rounds (compiled with -fmad=false:
// every bond's utilization, every K downdate equals the reference's for the same inputs).
//
// One round, after a converged solve (the host loop is svxg_cascade in capi.cu):
//   1. k_cascade_judge - every intact bond's load L (StressProblem::bond_load,
//      core/src/stress/stress.cpp:477-502), its utilization under lerp(judged, L, dif) when a
//      shock is on and the bond was judged before (World::Impl::judge,
//      core/src/world/world.cpp:1173-1201; lerp_load world_internal.hpp:452-461), else under L;
//      judged := L; a flag per bond at or over 1 and the largest utilization.
//   2. a scan and a scatter - the bonds over strength in index order.
//   3. k_cascade_select (one block) - the round's breaks (world.cpp:1219-1271): thr = max(1,
//      band x max phi), quota = max(1, (m + 3) / 4), K = min(max_breaks, max(#phi >= thr,
//      quota)); the K largest keys (phi descending, index ascending) by an exact radix select
//      on the 96-bit keys, sorted by a bitonic network.
//   4. remove_bonds_list - StressProblem::remove_bond (stress.cpp:260-284) of the list in
//      order, in parallel: every (bond, block) contribution links itself into its block's
//      chain; the last one to link walks the chain and applies the contributions in list order,
//      so each block gets the reference's subtractions in the reference's order.
//   5. detach - graph_components (world_internal.hpp:660-705) seeded by intact supports
//      (world.cpp:1371-1377) by lock-free union-find (hooks go from the larger root to the
//      smaller, so every chain ends); the nodes outside component 0 retire as
//      StressProblem::retire_nodes (stress.cpp:286-310) retires them: their bonds leave K in
//      bond order, then their rows become identities; their loads and motion become zero
//      (World::Impl::retire_structure_nodes, world.cpp:1460-1478).
#include <climits>

#include "blk6.cuh"
#include "problem.cuh"

namespace svxg {
namespace {

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

constexpr int kT = 256;
constexpr int kSelT = 1024;
constexpr int kSelShared = 2048;  // round breaks sorted in shared memory up to this many

unsigned grid_for(int64_t n, int t = kT) { return unsigned((n + t - 1) / t); }

// ---- 1. the judgement ----------------------------------------------------------------------

__global__ void k_cascade_judge(int32_t nb, const svxg_bond* __restrict__ bonds, const svxg_node* __restrict__ nodes,
                                const svxg_material* __restrict__ mats, const double* __restrict__ u,
                                double fragility, double dif, int blend, int skip_gone_a, svxg_bond_load* judged,
                                uint8_t* has, double* phi, uint8_t* mode, int32_t* flag, CascadeState* st) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  double ph = 0.0;
  if (k < nb && !bonds[k].broken && !(skip_gone_a && nodes[bonds[k].a].gone)) {
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
    svxg_bond_load Le = L;
    if (blend && judged && has[k]) {
      const svxg_bond_load J = judged[k];
      Le.N = J.N + dif * (L.N - J.N);
      Le.V1 = J.V1 + dif * (L.V1 - J.V1);
      Le.V2 = J.V2 + dif * (L.V2 - J.V2);
      Le.T = J.T + dif * (L.T - J.T);
      Le.M1 = J.M1 + dif * (L.M1 - J.M1);
      Le.M2 = J.M2 + dif * (L.M2 - J.M2);
    }
    uint8_t m = 0;
    ph = bond_utilization(b, Le, fragility, mats, &m);
    if (judged) {
      judged[k] = L;
      has[k] = 1;
    }
    if (mode) mode[k] = m;
    phi[k] = ph;
    flag[k] = ph >= 1.0 ? 1 : 0;
  } else if (k < nb) {
    phi[k] = 0.0;
    flag[k] = 0;
  }
  // the largest utilization: phi >= 0, so the bit patterns of the positive ones order as the
  // values do (the reference's max starts at 0 and never takes a NaN)
  unsigned long long bits = ph > 0.0 ? static_cast<unsigned long long>(__double_as_longlong(ph)) : 0ull;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, bits, d);
    bits = o > bits ? o : bits;
  }
  if ((threadIdx.x & 31) == 0 && bits) atomicMax(&st->maxphi_bits, bits);
}

__global__ void k_scatter_flagged(int32_t n, const int32_t* flag, const int32_t* pos, int32_t* out) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && flag[k]) out[pos[k]] = k;
}

__global__ void k_take_count(const int32_t* total, int32_t* dst) { *dst = *total; }

// ---- 3. the round's breaks ----------------------------------------------------------------

typedef unsigned __int128 u128;

// phi descending, then index ascending, as one unsigned key (larger first)
__device__ __forceinline__ u128 break_key(double ph, int32_t b) {
  return (u128(static_cast<unsigned long long>(__double_as_longlong(ph))) << 32) |
         u128(0xFFFFFFFFu - static_cast<uint32_t>(b));
}

__device__ __forceinline__ bool key_less(unsigned long long pa, int32_t ba, unsigned long long pb, int32_t bb) {
  return pa < pb || (pa == pb && ba > bb);  // (a smaller index is a larger key)
}

__device__ double block_max_d(double v, double* red) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, v, d);
    v = v < o ? o : v;
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < int(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      const double o = __shfl_xor_sync(0xffffffffu, v, d);
      v = v < o ? o : v;
    }
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  return red[0];
}

__device__ int32_t block_sum_i(int32_t v, int32_t* red) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < int(blockDim.x >> 5) ? red[lane] : 0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  return red[0];
}

// One block. over[0..m): the bonds over strength (m = st->m, set by the scan); sel[0..K): the
// bonds the round breaks, in the order the reference breaks them. gphi/gb: sort scratch of
// gcap entries (a power of two >= K) for rounds that break more than kSelShared bonds.
__global__ void __launch_bounds__(kSelT) k_cascade_select(const int32_t* over, const double* phi, double band,
                                                          int32_t max_breaks, BreakRule rule, const svxg_bond* bonds,
                                                          const uint8_t* mode, int32_t* sel,
                                                          unsigned long long* gphi, int32_t* gb, int64_t gcap,
                                                          CascadeState* st) {
  __shared__ double redd[32];
  __shared__ int32_t redi[32];
  __shared__ int32_t hist[256];
  __shared__ unsigned long long sphi[kSelShared];
  __shared__ int32_t sb[kSelShared];
  __shared__ int32_t s_digit, s_krem, s_fill;
  const int32_t m = st->m;
  if (m == 0) {
    if (threadIdx.x == 0) st->K = 0;
    return;
  }
  // the largest phi, the threshold, the bonds at or over it
  double top = 0.0;
  for (int32_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double v = phi[over[i]];
    top = top < v ? v : top;
  }
  top = block_max_d(top, redd);
  const double x = band * top;
  const double thr = 1.0 < x ? x : 1.0;
  int32_t c = 0;
  for (int32_t i = threadIdx.x; i < m; i += blockDim.x) c += phi[over[i]] >= thr ? 1 : 0;
  const int32_t n_thr = block_sum_i(c, redi);
  // the quota: a structure's round, at least the worst quarter (world.cpp:1258); a piece's, at
  // least ceil(fraction x m) (world_pieces.cpp:666)
  int64_t quota = rule.fraction < 0.0 ? max(int64_t(1), (int64_t(m) + 3) / 4)
                                      : static_cast<int64_t>(ceil(rule.fraction * static_cast<double>(m)));
  if (quota > m) quota = m;
  const int32_t take = max(n_thr, int32_t(quota));
  const int32_t K = min(max_breaks, take);
  // the K-th largest key, digit by digit from the top (12 bytes; keys are distinct)
  u128 prefix = 0;
  if (K < m) {
    if (threadIdx.x == 0) s_krem = K;
    for (int pos = 11; pos >= 0; --pos) {
      for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
      __syncthreads();
      const int hi_shift = 8 * (pos + 1);
      for (int32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const int32_t b = over[i];
        const u128 key = break_key(phi[b], b);
        if ((key >> hi_shift) == (prefix >> hi_shift)) atomicAdd(&hist[int((key >> (8 * pos)) & 0xFF)], 1);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int32_t krem = s_krem, cum = 0, d = 255;
        for (; d > 0; --d) {
          if (cum + hist[d] >= krem) break;
          cum += hist[d];
        }
        s_digit = d;
        s_krem = krem - cum;
      }
      __syncthreads();
      prefix |= u128(unsigned(s_digit)) << (8 * pos);
    }
  }
  // the selected keys (every key >= the K-th), then sorted
  int32_t P2 = 1;
  while (P2 < K) P2 <<= 1;
  const bool in_shared = P2 <= kSelShared;
  unsigned long long* kp = in_shared ? sphi : gphi;
  int32_t* kb = in_shared ? sb : gb;
  if (!in_shared && int64_t(P2) > gcap) {
    if (threadIdx.x == 0) st->K = -1;  // (the host sized the scratch for max_breaks: not reached)
    return;
  }
  if (threadIdx.x == 0) s_fill = 0;
  for (int32_t i = threadIdx.x; i < P2; i += blockDim.x) {
    kp[i] = 0ull;
    kb[i] = INT_MAX;
  }
  __syncthreads();
  for (int32_t i = threadIdx.x; i < m; i += blockDim.x) {
    const int32_t b = over[i];
    const double v = phi[b];
    if (K >= m || break_key(v, b) >= prefix) {
      const int32_t slot = atomicAdd(&s_fill, 1);
      kp[slot] = static_cast<unsigned long long>(__double_as_longlong(v));
      kb[slot] = b;
    }
  }
  __syncthreads();
  for (int32_t k = 2; k <= P2; k <<= 1) {
    for (int32_t j = k >> 1; j > 0; j >>= 1) {
      for (int32_t i = threadIdx.x; i < P2; i += blockDim.x) {
        const int32_t l = i ^ j;
        if (l > i) {
          const unsigned long long pa = kp[i], pb = kp[l];
          const int32_t ba = kb[i], bb = kb[l];
          // (i & k) == 0: this run ends larger-first
          const bool swap = (i & k) == 0 ? key_less(pa, ba, pb, bb) : key_less(pb, bb, pa, ba);
          if (swap) {
            kp[i] = pb;
            kp[l] = pa;
            kb[i] = bb;
            kb[l] = ba;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int32_t i = threadIdx.x; i < K; i += blockDim.x) sel[i] = kb[i];
  if (threadIdx.x == 0) {
    // an impact pays for its cracks in order: the first it cannot pay for ends the round
    // (world_pieces.cpp:672-683)
    int32_t keep = K, poor = 0;
    double spent = rule.spent;
    if (rule.energy >= 0.0) {
      for (int32_t t = 0; t < K; ++t) {
        const svxg_bond& B = bonds[kb[t]];
        const double crush = mode[kb[t]] == SVXG_FAIL_CRUSH ? rule.crush_energy : 1.0;
        const double g1 = rule.gf[B.ma], g2 = rule.gf[B.mb];
        const double cost = rule.fracture_energy * crush * B.area * mind(g1, g2) * B.strength;
        if (spent + cost > rule.energy) {
          keep = t;
          poor = 1;
          break;
        }
        spent += cost;
      }
    }
    st->K = keep;
    st->poor = poor;
    st->spent = spent;
    st->top = top;
    st->n_thr = n_thr;
  }
}

// ---- 4. bond removal in list order, in parallel -------------------------------------------------

__device__ __forceinline__ int64_t block_pos(const int32_t* rowptr, const int32_t* col, int32_t r, int32_t c) {
  for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
    if (col[k] == c) return k;
  return -1;
}

// contribution s = 4 t + j of list[t]: j = 0 K_aa, 1 K_bb, 2 K_ab, 3 K_ba
__global__ void k_rm_link(const int32_t* list, const int32_t* count_dev, int32_t count_host, const svxg_bond* bonds,
                          const uint8_t* in_k, const int32_t* dof, const int32_t* rowptr, const int32_t* col,
                          int32_t* head, int32_t* next, int64_t* tgt, CascadeState* st) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int32_t count = count_dev ? *count_dev : count_host;
  if (s >= 4 * int64_t(count)) return;
  const int32_t t = int32_t(s >> 2), j = int32_t(s & 3);
  const int32_t bi = list[t];
  tgt[s] = -1;
  if (!in_k[bi]) return;
  if (j == 0 && st) st->any_in_k = 1;
  const int32_t a = bonds[bi].a, bb = bonds[bi].b;
  const int32_t ia = dof[a];
  const int32_t ib = bb >= 0 ? dof[bb] : -1;
  const int32_t r = (j == 0 || j == 2) ? ia : ib;
  const int32_t c = (j == 0 || j == 3) ? ia : ib;
  if (r < 0 || c < 0) return;
  const int64_t pos = block_pos(rowptr, col, r, c);
  if (pos < 0) return;
  tgt[s] = pos;
  next[s] = atomicExch(&head[pos], int32_t(s));
}

__device__ void apply_contribution(int32_t s, const int32_t* list, const svxg_bond* bonds, const svxg_node* nodes,
                                   const svxg_material* mats, double* blk) {
  const int32_t j = s & 3;
  const svxg_bond b = bonds[list[s >> 2]];
  BondStiffness S;
  bond_stiffness(b, mats, S);
  const V3d p = v3of(b.p);
  const V3d ra = sub3(p, v3of(nodes[b.a].c));
  const V3d rb = b.b >= 0 ? sub3(p, v3of(nodes[b.b].c)) : V3d{0, 0, 0};
  if (j == 0) atbd_add_rigid_fast(ra, S, ra, -1.0, blk);
  else if (j == 1) atbd_add_rigid_fast(rb, S, rb, -1.0, blk);
  else if (j == 2) atbd_add_rigid_fast(ra, S, rb, 1.0, blk);
  else atbd_add_rigid_fast(rb, S, ra, 1.0, blk);
}

__global__ void k_rm_apply(const int32_t* list, const int32_t* count_dev, int32_t count_host, svxg_bond* bonds,
                           uint8_t* in_k, const svxg_node* nodes, const svxg_material* mats, double* val,
                           int32_t* head, const int32_t* next, const int64_t* tgt) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int32_t count = count_dev ? *count_dev : count_host;
  if (s >= 4 * int64_t(count)) return;
  const int64_t pos = tgt[s];
  if (pos >= 0 && __ldcg(&head[pos]) == int32_t(s)) {
    // the last contribution linked at this block: apply the chain in ascending order
    double* blk = val + 36 * pos;
    int32_t prev = -1;
    for (;;) {
      int32_t best = INT_MAX;
      for (int32_t q = int32_t(s); q >= 0; q = next[q])
        if (q > prev && q < best) best = q;
      if (best == INT_MAX) break;
      apply_contribution(best, list, bonds, nodes, mats, blk);
      prev = best;
    }
    head[pos] = -1;
  }
  if ((s & 3) == 0) {
    const int32_t bi = list[s >> 2];
    bonds[bi].broken = 1;
    bonds[bi].in_k = 0;
    in_k[bi] = 0;
  }
}

// block-Jacobi inverses of the diagonals the list touched (stress.cpp:276-282): of the final
// diagonal, which is what the reference's last recomputation of each sees
__global__ void k_rm_jinv(const int32_t* list, const int32_t* count_dev, int32_t count_host, const svxg_bond* bonds,
                          const int32_t* dof, const int32_t* rowptr, const double* val, const int64_t* tgt,
                          double* jinv, double id_scale) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int32_t count = count_dev ? *count_dev : count_host;
  if (s >= 2 * int64_t(count)) return;
  const int32_t t = int32_t(s >> 1), side = int32_t(s & 1);
  if (tgt[4 * int64_t(t) + side] < 0) return;  // (not in K, or no diagonal on this side)
  const int32_t bi = list[t];
  const int32_t nd = side == 0 ? bonds[bi].a : bonds[bi].b;
  const int32_t d = dof[nd];
  const double* D = val + 36 * int64_t(rowptr[d]);
  double tmp[36];
  double* J = jinv + 36 * int64_t(d);
  if (inv6(D, tmp)) {
    for (int q = 0; q < 36; ++q) J[q] = tmp[q];
  } else {
    for (int q = 0; q < 36; ++q) J[q] = (q % 7 == 0) ? 1.0 / id_scale : 0.0;
  }
}

// ---- 5. what no support holds ---------------------------------------------------------------------

__device__ __forceinline__ int32_t cc_find(const int32_t* parent, int32_t x) {
  // parents only ever point to smaller indices, so the walk ends; L2 reads see the hooks
  int32_t p = __ldcg(&parent[x]);
  while (p != x) {
    x = p;
    p = __ldcg(&parent[x]);
  }
  return x;
}

__global__ void k_cc_init(int32_t n, int32_t* parent, uint8_t* held, uint8_t* now) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  parent[i] = i;
  held[i] = 0;
  now[i] = 0;
}

__global__ void k_cc_hook(int32_t nb, const svxg_bond* bonds, int32_t* parent) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  if (bonds[k].broken || bonds[k].b < 0) return;
  int32_t x = bonds[k].a, y = bonds[k].b;
  for (;;) {
    x = cc_find(parent, x);
    y = cc_find(parent, y);
    if (x == y) return;
    if (x < y) {
      const int32_t t = x;
      x = y;
      y = t;
    }
    const int32_t old = atomicCAS(&parent[x], x, y);  // the larger root hooks under the smaller
    if (old == x) return;
    x = old;  // (hooked meanwhile: go on from where it went)
  }
}

__global__ void k_cc_flatten(int32_t n, int32_t* parent) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) parent[i] = cc_find(parent, i);
}

__global__ void k_cc_seed(int32_t nb, const svxg_bond* bonds, const int32_t* parent, uint8_t* held) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  if (!bonds[k].broken && bonds[k].b < 0) held[parent[bonds[k].a]] = 1;
}

__global__ void k_cc_loose(int32_t n, const svxg_node* nodes, const int32_t* parent, const uint8_t* held,
                           int32_t* flag) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (!nodes[i].gone && !held[parent[i]]) ? 1 : 0;
}

// retire_nodes' marks (stress.cpp:290-294) and the structure's zeroed loads and motion
__global__ void k_retire_mark(const int32_t* list, const int32_t* count, svxg_node* nodes, uint8_t* now,
                              const int32_t* dof, double* u, double* f, CascadeState* st) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *count) return;
  const int32_t i = list[t];
  nodes[i].gone = 1;
  now[i] = 1;
  for (int q = 0; q < 6; ++q) {
    u[6 * int64_t(i) + q] = 0.0;
    f[6 * int64_t(i) + q] = 0.0;
  }
  if (dof && dof[i] >= 0) st->r_dof = 1;
}

__global__ void k_retire_bond_flags(int32_t nb, const svxg_bond* bonds, const uint8_t* now, int32_t* flag) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int32_t a = bonds[k].a, b = bonds[k].b;
  flag[k] = (now[a] || (b >= 0 && now[b])) ? 1 : 0;
}

// retire_nodes' identity rows (stress.cpp:299-308), after its bond removals
__global__ void k_retire_rows(const int32_t* list, const int32_t* count, const int32_t* dof, const int32_t* rowptr,
                              double* val, double* jinv, int jacobi, double id_scale) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *count) return;
  const int32_t d = dof[list[t]];
  if (d < 0) return;
  double* D = val + 36 * int64_t(rowptr[d]);
  for (int q = 0; q < 36; ++q) D[q] = (q % 7 == 0) ? id_scale : 0.0;
  if (jacobi)
    for (int q = 0; q < 36; ++q) jinv[36 * int64_t(d) + q] = (q % 7 == 0) ? 1.0 / id_scale : 0.0;
}

// remove_bond on a problem not assembled: the bond only breaks (stress.cpp:262-263)
__global__ void k_mark_broken(const int32_t* list, const int32_t* count_dev, int32_t count_host, svxg_bond* bonds) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t count = count_dev ? *count_dev : count_host;
  if (t < count) bonds[list[t]].broken = 1;
}

__global__ void k_gather_modes(const int32_t* sel, int32_t count, const uint8_t* mode, uint8_t* out) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) out[t] = mode[sel[t]];
}

// bonds[list[t]].broken = 0: a caller's write to the public member (a chip's inner bonds keep
// their topology after the chip retires, world_pieces.cpp:800-802); in_k stays as it is
__global__ void k_unbreak(const int32_t* list, int32_t count, svxg_bond* bonds) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) bonds[list[t]].broken = 0;
}

__global__ void k_copy_flags(int32_t nb, const svxg_bond* bonds, const uint8_t* in_k_dev, uint8_t* broken,
                             uint8_t* in_k) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  broken[k] = bonds[k].broken;
  in_k[k] = in_k_dev ? in_k_dev[k] : 0;
}

template <class T>
T* carve(char*& p, size_t count) {
  T* r = reinterpret_cast<T*>(p);
  p += ((count * sizeof(T) + 255) / 256) * 256;
  return r;
}

}  // namespace

// the chains' heads: one per block of K, all -1 between calls
static int ensure_rm_head(Problem& P) {
  if (P.rm_head_cap >= P.K.nnzb && P.d_rm_head) return SVXG_OK;
  P.mem.release(P.d_rm_head);
  TRY(P.mem.alloc(&P.d_rm_head, size_t(std::max<int64_t>(P.K.nnzb, 1))));
  SVXG_CUDA(cudaMemsetAsync(P.d_rm_head, 0xFF, sizeof(int32_t) * size_t(std::max<int64_t>(P.K.nnzb, 1)), P.stream));
  P.rm_head_cap = std::max<int64_t>(P.K.nnzb, 1);
  return SVXG_OK;
}

int remove_bonds_list(Problem& P, const int32_t* list, const int32_t* count_dev, int32_t bound, CascadeState* st) {
  if (bound <= 0) return SVXG_OK;
  if (!P.assembled) {
    (k_mark_broken<<<grid_for(bound), kT, 0, P.stream>>>(list, count_dev, bound, P.d_bonds), SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaGetLastError());
    return SVXG_OK;
  }
  TRY(ensure_rm_head(P));
  char* base = nullptr;
  const size_t c4 = 4 * size_t(bound);
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&base), c4 * (sizeof(int32_t) + sizeof(int64_t)) + 1024,
                              P.stream));
  char* cur = base;
  int32_t* next = carve<int32_t>(cur, c4);
  int64_t* tgt = carve<int64_t>(cur, c4);
  const unsigned g4 = grid_for(int64_t(c4));
  (k_rm_link<<<g4, kT, 0, P.stream>>>(list, count_dev, bound, P.d_bonds, P.d_in_k, P.d_dof, P.K.rowptr, P.K.col,
                                      P.d_rm_head, next, tgt, st), SVXG_COUNT_LAUNCH());
  (k_rm_apply<<<g4, kT, 0, P.stream>>>(list, count_dev, bound, P.d_bonds, P.d_in_k, P.d_nodes, P.d_mats, P.K.val,
                                       P.d_rm_head, next, tgt), SVXG_COUNT_LAUNCH());
  if (P.jacobi_only && P.d_jinv)
    (k_rm_jinv<<<grid_for(2 * int64_t(bound)), kT, 0, P.stream>>>(list, count_dev, bound, P.d_bonds, P.d_dof,
                                                                 P.K.rowptr, P.K.val, tgt, P.d_jinv, P.id_scale),
     SVXG_COUNT_LAUNCH());
  cudaFreeAsync(base, P.stream);
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

int cascade_alloc(Problem& P, CascadeScratch& S, int32_t max_breaks) {
  const size_t n = size_t(std::max(P.n, 1)), nb = size_t(std::max(P.nb, 1));
  const size_t nf = std::max(n, nb);  // (flags: of bonds, then of nodes)
  int64_t p2 = 1;
  while (p2 < std::min<int64_t>(max_breaks, int64_t(nb))) p2 <<= 1;
  S.gcap = p2 > kSelShared ? p2 : 0;
  const size_t bytes = 256 * 40 + sizeof(CascadeState) + 3 * 6 * n * sizeof(double) + nb * sizeof(svxg_bond_load) +
                       nb * (1 + sizeof(double) + 4 * sizeof(int32_t)) + nf * sizeof(int32_t) + n * (2 + 3 * sizeof(int32_t)) +
                       size_t(S.gcap) * (sizeof(unsigned long long) + sizeof(int32_t)) + 4 * nb +
                       sizeof(double) * SVXG_MAX_MATERIALS;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&S.base), bytes, P.stream));
  S.stream = P.stream;
  char* c = S.base;
  S.st = carve<CascadeState>(c, 1);
  S.u = carve<double>(c, 6 * n);
  S.f = carve<double>(c, 6 * n);
  S.u0 = carve<double>(c, 6 * n);
  S.judged = carve<svxg_bond_load>(c, nb);
  S.has = carve<uint8_t>(c, nb);
  S.phi = carve<double>(c, nb);
  S.flag = carve<int32_t>(c, nf);
  S.pos = carve<int32_t>(c, nb);
  S.over = carve<int32_t>(c, nb);
  S.sel = carve<int32_t>(c, nb);
  S.blist = carve<int32_t>(c, nb);
  S.parent = carve<int32_t>(c, n);
  S.held = carve<uint8_t>(c, n);
  S.now = carve<uint8_t>(c, n);
  S.nlist = carve<int32_t>(c, n);
  S.npos = carve<int32_t>(c, n);
  S.gphi = carve<unsigned long long>(c, size_t(std::max<int64_t>(S.gcap, 1)));
  S.gb = carve<int32_t>(c, size_t(std::max<int64_t>(S.gcap, 1)));
  S.broken8 = carve<uint8_t>(c, nb);
  S.in_k8 = carve<uint8_t>(c, nb);
  S.mode = carve<uint8_t>(c, nb);
  S.selmode = carve<uint8_t>(c, nb);
  S.gf = carve<double>(c, SVXG_MAX_MATERIALS);
  return SVXG_OK;
}

void cascade_free(CascadeScratch& S) {
  if (S.base) cudaFreeAsync(S.base, S.stream);
  S.base = nullptr;
}

int cascade_judge(Problem& P, CascadeScratch& S, double fragility, double dif, int blend, double band,
                  int32_t max_breaks, const BreakRule& rule) {
  SVXG_CUDA(cudaMemsetAsync(S.st, 0, sizeof(CascadeState), P.stream));
  if (P.nb == 0) return SVXG_OK;
  const unsigned g = grid_for(P.nb);
  const bool piece = rule.fraction >= 0.0;  // (pieces: no judged loads; bonds of retired nodes skipped; modes kept)
  (k_cascade_judge<<<g, kT, 0, P.stream>>>(P.nb, P.d_bonds, P.d_nodes, P.d_mats, S.u, fragility, dif, blend,
                                           piece ? 1 : 0, piece ? nullptr : S.judged, S.has, S.phi, S.mode, S.flag,
                                           S.st), SVXG_COUNT_LAUNCH());
  TRY(exclusive_scan_i32(P, S.flag, S.pos, P.nb, nullptr));
  (k_scatter_flagged<<<g, kT, 0, P.stream>>>(P.nb, S.flag, S.pos, S.over), SVXG_COUNT_LAUNCH());
  (k_take_count<<<1, 1, 0, P.stream>>>(scan_total_device(P, P.nb), &S.st->m), SVXG_COUNT_LAUNCH());
  (k_cascade_select<<<1, kSelT, 0, P.stream>>>(S.over, S.phi, band, max_breaks, rule, P.d_bonds, S.mode, S.sel, S.gphi,
                                               S.gb, S.gcap, S.st), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

int cascade_find_loose(Problem& P, CascadeScratch& S) {
  if (P.n == 0) return SVXG_OK;
  const unsigned gn = grid_for(P.n), gb = grid_for(std::max(P.nb, 1));
  (k_cc_init<<<gn, kT, 0, P.stream>>>(P.n, S.parent, S.held, S.now), SVXG_COUNT_LAUNCH());
  if (P.nb > 0) (k_cc_hook<<<gb, kT, 0, P.stream>>>(P.nb, P.d_bonds, S.parent), SVXG_COUNT_LAUNCH());
  (k_cc_flatten<<<gn, kT, 0, P.stream>>>(P.n, S.parent), SVXG_COUNT_LAUNCH());
  if (P.nb > 0) (k_cc_seed<<<gb, kT, 0, P.stream>>>(P.nb, P.d_bonds, S.parent, S.held), SVXG_COUNT_LAUNCH());
  (k_cc_loose<<<gn, kT, 0, P.stream>>>(P.n, P.d_nodes, S.parent, S.held, S.flag), SVXG_COUNT_LAUNCH());
  TRY(exclusive_scan_i32(P, S.flag, S.npos, P.n, nullptr));
  (k_scatter_flagged<<<gn, kT, 0, P.stream>>>(P.n, S.flag, S.npos, S.nlist), SVXG_COUNT_LAUNCH());
  (k_take_count<<<1, 1, 0, P.stream>>>(scan_total_device(P, P.n), &S.st->r), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

int cascade_retire(Problem& P, CascadeScratch& S, int32_t r) {
  if (r <= 0) return SVXG_OK;
  const unsigned gr = grid_for(r);
  (k_retire_mark<<<gr, kT, 0, P.stream>>>(S.nlist, &S.st->r, P.d_nodes, S.now, P.assembled ? P.d_dof : nullptr, S.u,
                                          S.f, S.st), SVXG_COUNT_LAUNCH());
  if (P.nb > 0) {
    const unsigned gb = grid_for(P.nb);
    (k_retire_bond_flags<<<gb, kT, 0, P.stream>>>(P.nb, P.d_bonds, S.now, S.flag), SVXG_COUNT_LAUNCH());
    TRY(exclusive_scan_i32(P, S.flag, S.pos, P.nb, nullptr));
    (k_scatter_flagged<<<gb, kT, 0, P.stream>>>(P.nb, S.flag, S.pos, S.blist), SVXG_COUNT_LAUNCH());
    (k_take_count<<<1, 1, 0, P.stream>>>(scan_total_device(P, P.nb), &S.st->rb), SVXG_COUNT_LAUNCH());
    TRY(remove_bonds_list(P, S.blist, &S.st->rb, P.nb, S.st));
  }
  if (P.assembled)
    (k_retire_rows<<<gr, kT, 0, P.stream>>>(S.nlist, &S.st->r, P.d_dof, P.K.rowptr, P.K.val, P.d_jinv,
                                            P.jacobi_only ? 1 : 0, P.id_scale), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

int cascade_bond_flags(Problem& P, CascadeScratch& S) {
  if (P.nb == 0) return SVXG_OK;
  (k_copy_flags<<<grid_for(P.nb), kT, 0, P.stream>>>(P.nb, P.d_bonds, P.d_in_k, S.broken8, S.in_k8), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// union-find roots of the intact node-to-node bonds (each node's component's smallest index)
int cascade_roots(Problem& P, CascadeScratch& S) {
  if (P.n == 0) return SVXG_OK;
  const unsigned gn = grid_for(P.n), gb = grid_for(std::max(P.nb, 1));
  (k_cc_init<<<gn, kT, 0, P.stream>>>(P.n, S.parent, S.held, S.now), SVXG_COUNT_LAUNCH());
  if (P.nb > 0) (k_cc_hook<<<gb, kT, 0, P.stream>>>(P.nb, P.d_bonds, S.parent), SVXG_COUNT_LAUNCH());
  (k_cc_flatten<<<gn, kT, 0, P.stream>>>(P.n, S.parent), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

int cascade_gather_modes(Problem& P, CascadeScratch& S, int32_t count) {
  if (count <= 0) return SVXG_OK;
  (k_gather_modes<<<grid_for(count), kT, 0, P.stream>>>(S.sel, count, S.mode, S.selmode), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

int unbreak_list(Problem& P, const int32_t* list_dev, int32_t count) {
  if (count <= 0) return SVXG_OK;
  (k_unbreak<<<grid_for(count), kT, 0, P.stream>>>(list_dev, count, P.d_bonds), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

}  // namespace svxg
