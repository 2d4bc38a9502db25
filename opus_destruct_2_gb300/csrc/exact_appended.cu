// exact_appended.cu - nodes appended after an assemble: StressProblem::reassemble and
// extend_warm_start (core/src/stress/stress.cpp:178-244) on the device.
//
// reassemble: K again from the current graph. The multigrid built by the last assemble keeps
// preconditioning the first pc_n free nodes (its level-0 operator is the K of that assemble, so
// it is stale, as the reference's is); the appended nodes (free indices pc_n and up) get their own
// multigrid over K's appended diagonal block when there are at least 24 of them and it builds, else
// their block-Jacobi inverses - the two applied additively (stress.cpp:312-324).
//
// extend_warm_start: appended nodes take the rigid motion of their bonded, already known
// neighbours (u_c = u_a + th_a x (x_c - x_a)), averaged, for up to four passes; each node sums its
// bonds in bond order, as the reference's loop over the bonds does.
#include <algorithm>

#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 256;
inline unsigned nblk(int64_t n) { return unsigned((std::max<int64_t>(n, 1) + kT - 1) / kT); }

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

// free index -> index in the appended block (-1: not appended)
__global__ void k_sub_dof(int32_t n, const int32_t* dof, int32_t pc_n, int32_t* sub_dof) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sub_dof[i] = dof[i] >= pc_n ? dof[i] - pc_n : -1;
}

// blocks of appended row r (r >= pc_n) whose column is appended too
__global__ void k_sub_count(int32_t na, int32_t pc_n, const int32_t* rowptr, const int32_t* col, int32_t* len) {
  const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= na) return;
  int32_t c = 0;
  for (int32_t k = rowptr[pc_n + r]; k < rowptr[pc_n + r + 1]; ++k) c += col[k] >= pc_n ? 1 : 0;
  len[r] = c;
}

// the appended diagonal block (Bsr6Builder's order: the row's order in K, diagonal first)
__global__ void k_sub_fill(int32_t na, int32_t pc_n, const int32_t* rowptr, const int32_t* col, const double* val,
                           const int32_t* srow, int32_t* scol, double* sval) {
  const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= na) return;
  int32_t o = srow[r];
  for (int32_t k = rowptr[pc_n + r]; k < rowptr[pc_n + r + 1]; ++k) {
    if (col[k] < pc_n) continue;
    scol[o] = col[k] - pc_n;
    for (int q = 0; q < 36; ++q) sval[36 * int64_t(o) + q] = val[36 * int64_t(k) + q];
    ++o;
  }
}

__global__ void k_jacobi_rows(int32_t na, const double* __restrict__ jinv, const double* __restrict__ r,
                              double* __restrict__ z, const int32_t* stop) {
  if (stop && *stop) return;
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na) return;
  const double* J = jinv + 36 * int64_t(i);
  for (int a = 0; a < 6; ++a) {
    double s = 0.0;
    for (int c = 0; c < 6; ++c) s += J[6 * a + c] * r[6 * int64_t(i) + c];
    z[6 * int64_t(i) + a] = s;
  }
}

// ---- extend_warm_start ------------------------------------------------------------------------

// incident bonds of the appended nodes (intact, both ends nodes), counted
__global__ void k_inc_count(int32_t nb, const svxg_bond* bonds, int32_t first_new, int32_t* cnt) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const svxg_bond& b = bonds[k];
  if (b.broken || b.b < 0) return;
  if (b.a >= first_new) atomicAdd(&cnt[b.a - first_new], 1);
  if (b.b >= first_new) atomicAdd(&cnt[b.b - first_new], 1);
}

__global__ void k_inc_fill(int32_t nb, const svxg_bond* bonds, int32_t first_new, const int32_t* off, int32_t* cursor,
                           int32_t* list) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const svxg_bond& b = bonds[k];
  if (b.broken || b.b < 0) return;
  if (b.a >= first_new) list[off[b.a - first_new] + atomicAdd(&cursor[b.a - first_new], 1)] = k;
  if (b.b >= first_new) list[off[b.b - first_new] + atomicAdd(&cursor[b.b - first_new], 1)] = k;
}

// each appended node's list in bond order
__global__ void k_inc_sort(int32_t m, const int32_t* off, int32_t* list) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  for (int32_t u = off[i] + 1; u < off[i + 1]; ++u) {
    const int32_t v = list[u];
    int32_t c = u - 1;
    while (c >= off[i] && list[c] > v) {
      list[c + 1] = list[c];
      --c;
    }
    list[c + 1] = v;
  }
}

__global__ void k_known_init(int32_t n, int32_t first_new, const svxg_node* nodes, uint8_t* known) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) known[i] = (i < first_new && !nodes[i].gone) ? 1 : 0;
}

// one pass: appended node c, unknown at the pass start, averages the rigid transfers from its
// known neighbours (known_in: the pass start), then becomes known (known_out)
__global__ void k_extend_pass(int32_t n, int32_t first_new, const svxg_node* nodes, const svxg_bond* bonds,
                              const int32_t* off, const int32_t* list, const uint8_t* known_in, uint8_t* known_out,
                              double* u) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t c = first_new + j;
  if (c >= n) return;
  if (known_in[c]) {
    known_out[c] = 1;
    return;
  }
  double acc[6] = {0, 0, 0, 0, 0, 0};
  double w = 0.0;
  for (int32_t e = off[j]; e < off[j + 1]; ++e) {
    const svxg_bond& b = bonds[list[e]];
    const int32_t o = b.a == c ? b.b : b.a;
    if (!known_in[o]) continue;
    const svxg_v3 xc = nodes[c].c, xo = nodes[o].c;
    const double rx = xc.x - xo.x, ry = xc.y - xo.y, rz = xc.z - xo.z;
    const double* uo = u + 6 * int64_t(o);
    const double thx = uo[3], thy = uo[4], thz = uo[5];
    const double t[3] = {thy * rz - thz * ry, thz * rx - thx * rz, thx * ry - thy * rx};
    for (int q = 0; q < 3; ++q) acc[q] += uo[q] + t[q];
    for (int q = 3; q < 6; ++q) acc[q] += uo[q];
    w += 1.0;
  }
  known_out[c] = 0;
  if (w == 0.0) return;
  // (written after every node of the pass has read: the new values go to unknown nodes only,
  // which no node of this pass reads)
  for (int q = 0; q < 6; ++q) u[6 * int64_t(c) + q] = acc[q] / w;
  known_out[c] = 1;
}

}  // namespace

// the appended block's own multigrid (P.sub), or none when it does not build
int build_appended(Problem& P) {
  const int32_t na = P.nfree - P.pc_n;
  if (na < 24) return SVXG_OK;
  cudaStream_t st = P.stream;
  Problem* S = new Problem;
  S->device = P.device;
  S->stream = st;
  S->mem.stream = st;
  S->opt = P.opt;
  S->n = P.n;
  S->nb = 0;
  S->d_nodes = P.d_nodes;  // (borrowed: positions of the appended nodes)
  S->nfree = na;
  S->borrowed = true;
  S->h_s = P.h_s;
  int e = S->mem.alloc(&S->d_dof, size_t(std::max(P.n, 1)));
  if (!e) {
    (k_sub_dof<<<nblk(P.n), kT, 0, st>>>(P.n, P.d_dof, P.pc_n, S->d_dof), SVXG_COUNT_LAUNCH());
    e = S->mem.alloc(&S->K.rowptr, size_t(na) + 1);
  }
  int32_t* len = nullptr;
  if (!e) e = S->mem.alloc(&len, size_t(na) + 1);
  int32_t snnz = 0;
  if (!e) {
    // (len[na] = 0: the scan's total is then the block count)
    if (cudaMemsetAsync(len, 0, sizeof(int32_t) * (size_t(na) + 1), st) != cudaSuccess) e = SVXG_ERR_CUDA;
    (k_sub_count<<<nblk(na), kT, 0, st>>>(na, P.pc_n, P.K.rowptr, P.K.col, len), SVXG_COUNT_LAUNCH());
    e = exclusive_scan_i32(P, len, S->K.rowptr, int64_t(na) + 1, &snnz);
  }
  if (!e) e = S->mem.alloc(&S->K.col, size_t(snnz));
  if (!e) e = S->mem.alloc(&S->K.val, 36 * size_t(snnz));
  if (!e) {
    S->K.n = na;
    S->K.nnzb = snnz;
    (k_sub_fill<<<nblk(na), kT, 0, st>>>(na, P.pc_n, P.K.rowptr, P.K.col, P.K.val, S->K.rowptr, S->K.col, S->K.val),
     SVXG_COUNT_LAUNCH());
    if (cudaGetLastError() != cudaSuccess) e = SVXG_ERR_CUDA;
  }
  if (len) S->mem.release(len);
  int32_t built = 0;
  if (!e) e = build_multigrid(*S, &built);
  if (e || !built) {
    S->mem.release_all();
    delete S;
    return e;
  }
  P.sub = S;
  return SVXG_OK;
}

void release_appended(Problem& P) {
  if (!P.sub) return;
  Problem* S = P.sub;
  S->stream = P.stream;
  S->mem.stream = P.stream;
  S->mem.release_all();
  delete S;
  P.sub = nullptr;
}

// z = M^-1 r over the free nodes: the multigrid of the last assemble on its pc_n nodes, and the
// appended nodes' own multigrid or block-Jacobi inverses on the rest (additive)
int precondition_amg(Problem& P, const double* r, double* z) {
  TRY(vcycle(P, r, z));
  if (P.pc_n >= P.nfree) return SVXG_OK;
  const int32_t na = P.nfree - P.pc_n;
  const size_t o = 6 * size_t(P.pc_n);
  if (P.sub) {
    Problem& S = *P.sub;
    S.stream = P.stream;
    S.mem.stream = P.stream;
    S.cycle_stop = P.cycle_stop;
    return vcycle(S, r + o, z + o);
  }
  (k_jacobi_rows<<<nblk(na), kT, 0, P.stream>>>(na, P.d_jinv + 36 * size_t(P.pc_n), r + o, z + o, P.cycle_stop),
   SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

// u: device, 6 per node (node order); nodes first_new.. are the appended ones
int extend_warm_start_device(Problem& P, double* u, int32_t first_new) {
  const int32_t n = P.n, nb = P.nb;
  if (first_new >= n || first_new < 0) return SVXG_OK;
  cudaStream_t st = P.stream;
  const int32_t m = n - first_new;
  int32_t *cnt = nullptr, *off = nullptr, *cursor = nullptr, *list = nullptr;
  uint8_t* known = nullptr;
  TRY(P.mem.alloc(&cnt, size_t(m) + 1));
  TRY(P.mem.alloc(&off, size_t(m) + 1));
  TRY(P.mem.alloc(&cursor, size_t(m) + 1));
  TRY(P.mem.alloc(&known, 2 * size_t(n)));
  SVXG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t(m) + 1), st));
  SVXG_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t(m) + 1), st));
  if (nb > 0) (k_inc_count<<<nblk(nb), kT, 0, st>>>(nb, P.d_bonds, first_new, cnt), SVXG_COUNT_LAUNCH());
  int32_t total = 0;
  int e = exclusive_scan_i32(P, cnt, off, int64_t(m) + 1, &total);
  if (!e) e = P.mem.alloc(&list, size_t(total));
  if (!e) {
    if (nb > 0) (k_inc_fill<<<nblk(nb), kT, 0, st>>>(nb, P.d_bonds, first_new, off, cursor, list), SVXG_COUNT_LAUNCH());
    (k_inc_sort<<<nblk(m), kT, 0, st>>>(m, off, list), SVXG_COUNT_LAUNCH());
    (k_known_init<<<nblk(n), kT, 0, st>>>(n, first_new, P.d_nodes, known), SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaMemcpyAsync(known + n, known, size_t(n), cudaMemcpyDeviceToDevice, st));
    for (int pass = 0; pass < 4; ++pass) {
      const uint8_t* kin = known + (pass & 1 ? n : 0);
      uint8_t* kout = known + (pass & 1 ? 0 : n);
      (k_extend_pass<<<nblk(m), kT, 0, st>>>(n, first_new, P.d_nodes, P.d_bonds, off, list, kin, kout, u),
       SVXG_COUNT_LAUNCH());
      // (nodes before first_new keep their flags in both halves: copied above)
    }
    if (cudaGetLastError() != cudaSuccess) e = SVXG_ERR_CUDA;
  }
  P.mem.release(cnt);
  P.mem.release(off);
  P.mem.release(cursor);
  P.mem.release(known);
  if (list) P.mem.release(list);
  return e;
}

}  // namespace svxg
