// exact_assemble.cu - K from the bonds on the device, value for value the reference's K.
//
// Restates StressProblem::build_matrix (core/src/stress/stress.cpp:84-132) with Bsr6Builder's
// layout (core/src/solve/amg.cpp:185-224) as parallel passes:
//   1. DOF numbering: free nodes in node order (a scan of the free flags);
//   2. per free node, its intact bonds ("incidences") gathered and sorted two ways: by bond index
//      (the order the reference adds a node's diagonal contributions in) and by (neighbour,
//      bond index) (the order of each off-diagonal block's contributions);
//   3. row lengths = 1 + distinct free neighbours, a scan for rowptr, columns diagonal first then
//      ascending (Bsr6Builder::finish's order);
//   4. one thread per block sums its contributions in bond order: the same additions, in the
//      same order, as the reference's sequential loop over bonds (this file is compiled with
//      -fmad=false: no contraction, IEEE division and square root);
//   5. id_scale (the mean diagonal translation stiffness) summed row by row in order, and retired
//      or empty rows set to id_scale I.
// No floating-point atomics anywhere: K is identical run to run and equal to the reference's.
#include "blk6.cuh"
#include "exact_sum.cuh"
#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;
inline unsigned blocks_for(int64_t n, int t = kT) { return unsigned((n + t - 1) / t); }

__global__ void k_free_flags(int32_t n, const svxg_node* nodes, int32_t* flags) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = nodes[i].fixed ? 0 : 1;
}

__global__ void k_dof(int32_t n, const svxg_node* nodes, const int32_t* scan, int32_t* dof, int32_t* node_of_dof) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t d = nodes[i].fixed ? -1 : scan[i];
  dof[i] = d;
  if (d >= 0) node_of_dof[d] = i;
}

// in_k flags (stress.cpp:95-99) and incidence counts of free endpoints
__global__ void k_classify(int32_t nb, const svxg_bond* bonds, const svxg_node* nodes, const int32_t* dof,
                           uint8_t* in_k, int32_t* cnt) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const svxg_bond& b = bonds[k];
  const bool ik = !b.broken && !nodes[b.a].gone && !(b.b >= 0 && nodes[b.b].gone);
  in_k[k] = ik ? 1 : 0;
  if (!ik) return;
  if (dof[b.a] >= 0) atomicAdd(&cnt[b.a], 1);
  if (b.b >= 0 && dof[b.b] >= 0) atomicAdd(&cnt[b.b], 1);
}

// incidence entries: high word = neighbour's free index + 1 (0: support or fixed neighbour),
// low word = 2 bond + side (side 1: this node is the bond's b)
__global__ void k_fill(int32_t nb, const svxg_bond* bonds, const int32_t* dof, const uint8_t* in_k, const int32_t* off,
                       int32_t* cursor, uint64_t* by_nbr) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb || !in_k[k]) return;
  const svxg_bond& b = bonds[k];
  const int32_t da = dof[b.a];
  const int32_t db = b.b >= 0 ? dof[b.b] : -1;
  if (da >= 0) {
    const int32_t s = atomicAdd(&cursor[b.a], 1);
    by_nbr[off[b.a] + s] = (uint64_t(uint32_t(db + 1)) << 32) | uint32_t(2 * k);
  }
  if (db >= 0) {
    const int32_t s = atomicAdd(&cursor[b.b], 1);
    by_nbr[off[b.b] + s] = (uint64_t(uint32_t(da + 1)) << 32) | uint32_t(2 * k + 1);
  }
}

// per node: sort its entries by (neighbour, bond) and a copy by bond; count its row's blocks
__global__ void k_sort_rows(int32_t n, const int32_t* dof, const int32_t* off, uint64_t* by_nbr, uint32_t* by_bond,
                            int32_t* rowlen) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || dof[i] < 0) return;
  const int32_t e0 = off[i], e1 = off[i + 1];
  for (int32_t a = e0 + 1; a < e1; ++a) {
    const uint64_t v = by_nbr[a];
    int32_t c = a - 1;
    while (c >= e0 && by_nbr[c] > v) {
      by_nbr[c + 1] = by_nbr[c];
      --c;
    }
    by_nbr[c + 1] = v;
  }
  for (int32_t a = e0; a < e1; ++a) by_bond[a] = uint32_t(by_nbr[a]);
  for (int32_t a = e0 + 1; a < e1; ++a) {
    const uint32_t v = by_bond[a];
    int32_t c = a - 1;
    while (c >= e0 && by_bond[c] > v) {
      by_bond[c + 1] = by_bond[c];
      --c;
    }
    by_bond[c + 1] = v;
  }
  int32_t distinct = 0;
  uint32_t prev = 0;
  for (int32_t a = e0; a < e1; ++a) {
    const uint32_t nb1 = uint32_t(by_nbr[a] >> 32);
    if (nb1 != 0 && nb1 != prev) ++distinct;
    prev = nb1;
  }
  rowlen[dof[i]] = 1 + distinct;
}

// columns and each block's contribution range: the diagonal's in by_bond, the others' in by_nbr
__global__ void k_columns(int32_t nfree, const int32_t* node_of_dof, const int32_t* off, const uint64_t* by_nbr,
                          const int32_t* rowptr, int32_t* col, int32_t* cstart, int32_t* ccount) {
  const int32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nfree) return;
  const int32_t i = node_of_dof[d];
  const int32_t e0 = off[i], e1 = off[i + 1];
  int32_t k = rowptr[d];
  col[k] = d;
  cstart[k] = e0;
  ccount[k] = e1 - e0;
  ++k;
  int32_t a = e0;
  while (a < e1) {
    const uint32_t nb1 = uint32_t(by_nbr[a] >> 32);
    int32_t z = a + 1;
    while (z < e1 && uint32_t(by_nbr[z] >> 32) == nb1) ++z;
    if (nb1 != 0) {
      col[k] = int32_t(nb1) - 1;
      cstart[k] = a;
      ccount[k] = z - a;
      ++k;
    }
    a = z;
  }
}

__device__ __forceinline__ V3d node_c(const svxg_node* nodes, int32_t i) { return v3of(nodes[i].c); }

// one thread per block: its contributions in bond order (stress.cpp:94-109)
// DIAG: a thread per row, its diagonal block (the row's first: every bond of the node); else a
// thread per block, the off-diagonal ones (one bond each, as a rule). The two kinds take separate
// launches: a diagonal block sums several bonds, and mixed in one warp it would hold the warp's
// other lanes idle on the FP64 pipe.
template <bool DIAG>
__global__ void k_block_values(int64_t nnzb, int32_t nfree, const int32_t* rowptr, const int32_t* col,
                               const int32_t* node_of_dof, const int32_t* cstart, const int32_t* ccount,
                               const uint64_t* by_nbr, const uint32_t* by_bond, const svxg_bond* bonds,
                               const svxg_node* nodes, const svxg_material* mats, double* val) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  int32_t d;
  int64_t k;
  if (DIAG) {
    if (t >= nfree) return;
    d = int32_t(t);
    k = rowptr[d];
  } else {
    if (t >= nnzb) return;
    k = t;
    // the block's row: binary search in rowptr
    int32_t lo = 0, hi = nfree - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) >> 1;
      if (rowptr[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    d = lo;
    if (rowptr[d] == k) return;  // (the diagonal: the DIAG launch)
  }
  const bool diag = DIAG;
  const int32_t i = node_of_dof[d];
  double C[36];
  for (int q = 0; q < 36; ++q) C[q] = 0.0;
  const int32_t e0 = cstart[k], e1 = e0 + ccount[k];
  for (int32_t e = e0; e < e1; ++e) {
    const uint32_t code = diag ? by_bond[e] : uint32_t(by_nbr[e]);
    const int32_t bi = int32_t(code >> 1);
    const int side = int(code & 1u);
    const svxg_bond b = bonds[bi];
    BondStiffness S;
    bond_stiffness(b, mats, S);
    const V3d p = v3of(b.p);
    const V3d rs = sub3(p, node_c(nodes, i));
    if (diag) {
      atbd_add_rigid_fast(rs, S, rs, 1.0, C);
    } else {
      const int32_t other = side ? b.a : b.b;
      const V3d ro = sub3(p, node_c(nodes, other));
      atbd_add_rigid_fast(rs, S, ro, -1.0, C);
    }
  }
  double* out = val + 36 * k;
  for (int q = 0; q < 36; ++q) out[q] = C[q];
  (void)col;
}

// per row: the diagonal's translational trace / 3 when positive (the id_scale terms), and
// whether the row becomes an identity (retired node or empty diagonal)
__global__ void k_trace(int32_t nfree, const int32_t* rowptr, const double* val, const int32_t* node_of_dof,
                        const svxg_node* nodes, double* term, uint8_t* ident, int32_t* nident) {
  const int32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nfree) return;
  const double* D = val + 36 * int64_t(rowptr[d]);
  const double t = D[0] + D[7] + D[14];
  term[d] = t > 0 ? t / 3.0 : -1.0;
  const bool empty = D[0] == 0.0 && D[7] == 0.0 && D[14] == 0.0;
  const bool id = nodes[node_of_dof[d]].gone || empty;
  ident[d] = id ? 1 : 0;
  if (id) atomicAdd(nident, 1);
}

// id_scale (stress.cpp:112-122): the rows' terms summed one after another, in row order (the
// sequential sum's exact bits, computed in parallel: exact_sum.cuh), over their count
__global__ void __launch_bounds__(exact::kThreads) k_id_scale(int32_t nfree, const double* term, double* out) {
  const auto f = [term](int64_t d) {
    const double t = term[d];
    return t >= 0.0 ? t : 0.0;
  };
  // (one warp for a short sum: launched with 32 threads)
  const double tr = blockDim.x == 32 ? exact::warp_sequential_sum_from(0.0, 0, nfree, f)
                                     : exact::sequential_sum(nfree, f);
  __shared__ int32_t cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int32_t c = 0;
  for (int32_t d = threadIdx.x; d < nfree; d += blockDim.x) c += term[d] >= 0.0 ? 1 : 0;
  atomicAdd(&cnt, c);
  __syncthreads();
  if (threadIdx.x == 0) out[0] = cnt ? tr / cnt : 1.0;
}

// retired and empty rows: id_scale on the diagonal (stress.cpp:123-130)
__global__ void k_identity(int32_t nfree, const int32_t* rowptr, const uint8_t* ident, const double* id_scale,
                           double* val) {
  const int32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nfree || !ident[d]) return;
  double* D = val + 36 * int64_t(rowptr[d]);
  const double s = *id_scale;
  for (int q = 0; q < 6; ++q) D[q * 7] = s;
}

// block-Jacobi inverses (stress.cpp:152-157)
__global__ void k_jacobi(int32_t nfree, const int32_t* rowptr, const double* val, double id_scale, double* jinv) {
  const int32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nfree) return;
  const double* D = val + 36 * int64_t(rowptr[d]);
  double* J = jinv + 36 * int64_t(d);
  double tmp[36];
  if (inv6(D, tmp)) {
    for (int q = 0; q < 36; ++q) J[q] = tmp[q];
  } else {
    for (int q = 0; q < 36; ++q) J[q] = (q % 7 == 0) ? 1.0 / id_scale : 0.0;
  }
}

__device__ double* find_block(const int32_t* rowptr, const int32_t* col, double* val, int32_t r, int32_t c) {
  for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
    if (col[k] == c) return val + 36 * int64_t(k);
  return nullptr;
}

// StressProblem::remove_bond (stress.cpp:260-284) for a list of bonds, one after another (a block
// touched by two of them gets the two subtractions in list order, as the reference's calls do).
__global__ void k_remove_bonds(const int32_t* list, int32_t count, svxg_bond* bonds, uint8_t* in_k,
                               const svxg_node* nodes, const svxg_material* mats, const int32_t* dof,
                               const int32_t* rowptr, const int32_t* col, double* val, double* jinv, int jacobi,
                               double id_scale) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int32_t t = 0; t < count; ++t) {
    const int32_t bi = list[t];
    svxg_bond& b = bonds[bi];
    b.broken = 1;
    if (!in_k[bi]) continue;
    in_k[bi] = 0;
    b.in_k = 0;
    BondStiffness S;
    bond_stiffness(b, mats, S);
    const V3d p = v3of(b.p);
    const int32_t ia = dof[b.a];
    const int32_t ib = b.b >= 0 ? dof[b.b] : -1;
    const V3d ra = sub3(p, v3of(nodes[b.a].c));
    const V3d rb = b.b >= 0 ? sub3(p, v3of(nodes[b.b].c)) : V3d{0, 0, 0};
    if (ia >= 0) atbd_add_rigid_fast(ra, S, ra, -1.0, find_block(rowptr, col, val, ia, ia));
    if (ib >= 0) atbd_add_rigid_fast(rb, S, rb, -1.0, find_block(rowptr, col, val, ib, ib));
    if (ia >= 0 && ib >= 0) {
      if (double* k1 = find_block(rowptr, col, val, ia, ib)) atbd_add_rigid_fast(ra, S, rb, 1.0, k1);
      if (double* k2 = find_block(rowptr, col, val, ib, ia)) atbd_add_rigid_fast(rb, S, ra, 1.0, k2);
    }
    if (jacobi) {
      const int32_t ds[2] = {ia, ib};
      for (int u = 0; u < 2; ++u) {
        const int32_t d = ds[u];
        if (d < 0) continue;
        const double* D = val + 36 * int64_t(rowptr[d]);
        double tmp[36];
        double* J = jinv + 36 * int64_t(d);
        if (inv6(D, tmp)) {
          for (int q = 0; q < 36; ++q) J[q] = tmp[q];
        } else {
          for (int q = 0; q < 36; ++q) J[q] = (q % 7 == 0) ? 1.0 / id_scale : 0.0;
        }
      }
    }
  }
}

// retire_nodes' identity rows (stress.cpp:299-308)
__global__ void k_identity_rows(const int32_t* rows, int32_t count, const int32_t* rowptr, double* val, double* jinv,
                                int jacobi, double id_scale) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int32_t d = rows[t];
  double* D = val + 36 * int64_t(rowptr[d]);
  for (int q = 0; q < 36; ++q) D[q] = (q % 7 == 0) ? id_scale : 0.0;
  if (jacobi)
    for (int q = 0; q < 36; ++q) jinv[36 * int64_t(d) + q] = (q % 7 == 0) ? 1.0 / id_scale : 0.0;
}

template <class T>
struct Tmp {
  T* p = nullptr;
  cudaStream_t s;
  Tmp(cudaStream_t st) : s(st) {}
  int alloc(size_t n) {
    cudaError_t e = pool_malloc_async(reinterpret_cast<void**>(&p), (n ? n : 1) * sizeof(T), s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(std::string("device allocation: ") + cudaGetErrorString(e));
      p = nullptr;
      return e == cudaErrorMemoryAllocation ? SVXG_ERR_NOMEM : SVXG_ERR_CUDA;
    }
    return SVXG_OK;
  }
  ~Tmp() {
    if (p) cudaFreeAsync(p, s);
  }
};

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

}  // namespace

int assemble_matrix(Problem& P) {
  cudaStream_t st = P.stream;
  const int32_t n = P.n, nb = P.nb;
  // 1. DOF numbering
  Tmp<int32_t> flags(st), scan(st), node_of_dof(st);
  TRY(flags.alloc(size_t(n)));
  TRY(scan.alloc(size_t(n)));
  TRY(node_of_dof.alloc(size_t(n)));
  P.mem.release(P.d_dof);
  TRY(P.mem.alloc(&P.d_dof, size_t(n)));
  if (n > 0) (k_free_flags<<<blocks_for(n), kT, 0, st>>>(n, P.d_nodes, flags.p), SVXG_COUNT_LAUNCH());
  int32_t nfree = 0;
  TRY(exclusive_scan_i32(P, flags.p, scan.p, n, &nfree));
  if (n > 0) (k_dof<<<blocks_for(n), kT, 0, st>>>(n, P.d_nodes, scan.p, P.d_dof, node_of_dof.p), SVXG_COUNT_LAUNCH());
  P.nfree = nfree;
  trace_mark(P, "assemble: DOF numbering");
  // 2. incidences
  P.mem.release(P.d_in_k);
  TRY(P.mem.alloc(&P.d_in_k, size_t(nb)));
  Tmp<int32_t> cnt(st), off(st), cursor(st);
  TRY(cnt.alloc(size_t(n) + 1));
  TRY(off.alloc(size_t(n) + 1));
  TRY(cursor.alloc(size_t(n) + 1));
  SVXG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (size_t(n) + 1), st));
  SVXG_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * (size_t(n) + 1), st));
  if (nb > 0) (k_classify<<<blocks_for(nb), kT, 0, st>>>(nb, P.d_bonds, P.d_nodes, P.d_dof, P.d_in_k, cnt.p), SVXG_COUNT_LAUNCH());
  int32_t ninc = 0;
  TRY(exclusive_scan_i32(P, cnt.p, off.p, int64_t(n) + 1, &ninc));
  Tmp<uint64_t> by_nbr(st);
  Tmp<uint32_t> by_bond(st);
  TRY(by_nbr.alloc(size_t(ninc)));
  TRY(by_bond.alloc(size_t(ninc)));
  if (nb > 0) (k_fill<<<blocks_for(nb), kT, 0, st>>>(nb, P.d_bonds, P.d_dof, P.d_in_k, off.p, cursor.p, by_nbr.p), SVXG_COUNT_LAUNCH());
  trace_mark(P, "assemble: incidences");
  // 3. pattern
  Tmp<int32_t> rowlen(st);
  TRY(rowlen.alloc(size_t(nfree) + 1));
  SVXG_CUDA(cudaMemsetAsync(rowlen.p, 0, sizeof(int32_t) * (size_t(nfree) + 1), st));
  if (n > 0) (k_sort_rows<<<blocks_for(n, 128), 128, 0, st>>>(n, P.d_dof, off.p, by_nbr.p, by_bond.p, rowlen.p), SVXG_COUNT_LAUNCH());
  P.mem.release(P.K.rowptr);
  TRY(P.mem.alloc(&P.K.rowptr, size_t(nfree) + 1));
  int32_t nnzb = 0;
  TRY(exclusive_scan_i32(P, rowlen.p, P.K.rowptr, int64_t(nfree) + 1, &nnzb));
  P.K.n = nfree;
  P.K.nnzb = nnzb;
  P.mem.release(P.K.col);
  P.mem.release(P.K.val);
  P.mem.release(P.K.val32);
  TRY(P.mem.alloc(&P.K.col, size_t(nnzb)));
  TRY(P.mem.alloc(&P.K.val, size_t(nnzb) * 36));
  Tmp<int32_t> cstart(st), ccount(st);
  TRY(cstart.alloc(size_t(nnzb)));
  TRY(ccount.alloc(size_t(nnzb)));
  if (nfree > 0)
    (k_columns<<<blocks_for(nfree), kT, 0, st>>>(nfree, node_of_dof.p, off.p, by_nbr.p, P.K.rowptr, P.K.col, cstart.p,
                                                ccount.p), SVXG_COUNT_LAUNCH());
  trace_mark(P, "assemble: pattern");
  // 4. values
  if (nnzb > 0) {
    (k_block_values<true><<<blocks_for(nfree, 128), 128, 0, st>>>(nnzb, nfree, P.K.rowptr, P.K.col, node_of_dof.p,
                                                                 cstart.p, ccount.p, by_nbr.p, by_bond.p, P.d_bonds,
                                                                 P.d_nodes, P.d_mats, P.K.val), SVXG_COUNT_LAUNCH());
    (k_block_values<false><<<blocks_for(nnzb, 128), 128, 0, st>>>(nnzb, nfree, P.K.rowptr, P.K.col, node_of_dof.p,
                                                                  cstart.p, ccount.p, by_nbr.p, by_bond.p, P.d_bonds,
                                                                  P.d_nodes, P.d_mats, P.K.val), SVXG_COUNT_LAUNCH());
  }
  trace_mark(P, "assemble: block values");
  // 5. id_scale and identity rows
  Tmp<double> term(st), ids(st);
  Tmp<uint8_t> ident(st);
  Tmp<int32_t> nident(st);
  TRY(term.alloc(size_t(nfree)));
  TRY(ident.alloc(size_t(nfree)));
  TRY(nident.alloc(1));
  TRY(ids.alloc(1));
  SVXG_CUDA(cudaMemsetAsync(nident.p, 0, sizeof(int32_t), st));
  if (nfree > 0)
    (k_trace<<<blocks_for(nfree), kT, 0, st>>>(nfree, P.K.rowptr, P.K.val, node_of_dof.p, P.d_nodes, term.p, ident.p,
                                              nident.p), SVXG_COUNT_LAUNCH());
  (k_id_scale<<<1, nfree <= exact::kWarpSumMax ? 32 : exact::kThreads, 0, st>>>(nfree, term.p, ids.p),
   SVXG_COUNT_LAUNCH());
  if (nfree > 0) (k_identity<<<blocks_for(nfree), kT, 0, st>>>(nfree, P.K.rowptr, ident.p, ids.p, P.K.val), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  SVXG_CUDA(cudaMemcpyAsync(&P.id_scale, ids.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  P.h_dof.resize(size_t(n));
  if (n > 0) SVXG_CUDA(cudaMemcpyAsync(P.h_dof.data(), P.d_dof, sizeof(int32_t) * size_t(n), cudaMemcpyDeviceToHost, st));
  P.h_in_k.resize(static_cast<size_t>(nb));
  if (nb > 0) SVXG_CUDA(cudaMemcpyAsync(P.h_in_k.data(), P.d_in_k, size_t(nb), cudaMemcpyDeviceToHost, st));
  SVXG_CUDA(host_wait(st));
  return SVXG_OK;
}

int build_jacobi(Problem& P) {
  P.mem.release(P.d_jinv);
  TRY(P.mem.alloc(&P.d_jinv, size_t(P.nfree) * 36));
  if (P.nfree > 0)
    (k_jacobi<<<blocks_for(P.nfree), kT, 0, P.stream>>>(P.nfree, P.K.rowptr, P.K.val, P.id_scale, P.d_jinv), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// up to this many bonds, one thread removes them one after another (one launch)
constexpr int32_t kSequentialRemoveMax = 4;

int remove_bonds_device(Problem& P, const int32_t* list, int32_t count) {
  if (count <= 0) return SVXG_OK;
  Tmp<int32_t> d(P.stream);
  TRY(d.alloc(size_t(count)));
  SVXG_CUDA(cudaMemcpyAsync(d.p, list, sizeof(int32_t) * size_t(count), cudaMemcpyHostToDevice, P.stream));
  if (count > kSequentialRemoveMax) {  // (many: every block's chain in parallel, the same bits)
    TRY(remove_bonds_list(P, d.p, nullptr, count, nullptr));
    SVXG_CUDA(host_wait(P.stream));
    return SVXG_OK;
  }
  (k_remove_bonds<<<1, 1, 0, P.stream>>>(d.p, count, P.d_bonds, P.d_in_k, P.d_nodes, P.d_mats, P.d_dof, P.K.rowptr,
                                        P.K.col, P.K.val, P.d_jinv, P.jacobi_only ? 1 : 0, P.id_scale), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

int set_identity_rows(Problem& P, const int32_t* rows, int32_t count) {
  if (count <= 0) return SVXG_OK;
  Tmp<int32_t> d(P.stream);
  TRY(d.alloc(size_t(count)));
  SVXG_CUDA(cudaMemcpyAsync(d.p, rows, sizeof(int32_t) * size_t(count), cudaMemcpyHostToDevice, P.stream));
  (k_identity_rows<<<blocks_for(count), kT, 0, P.stream>>>(d.p, count, P.K.rowptr, P.K.val, P.d_jinv,
                                                         P.jacobi_only ? 1 : 0, P.id_scale), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

}  // namespace svxg
