// spmv_row.cuh - the warp-per-block-row product of a 6x6 BSR matrix, shared by every SpMV.
//
// One warp owns one block row. Lanes 6g + c (g < 5, c < 6) take row c of every fifth block; the
// row's column indices arrive first, in one coalesced load (lane j holds the j-th block's column,
// broadcast by shuffles), and each group issues the loads of two blocks (k and k + 5: six
// 8-byte or 16-byte value loads and six broadcast x loads) before it multiplies, so a row of up
// to ten blocks costs one dependent round trip after the column indices. The five groups' sums
// meet in lanes 0-5.
#pragma once

#include <cstdint>

namespace svxg {

template <typename V>
struct Vec2;
template <>
struct Vec2<float> {
  using T = float2;
};
template <>
struct Vec2<double> {
  using T = double2;
};

// Rows of a batch (many graphs as one block-diagonal problem, every level of its multigrid block
// diagonal too) whose graph's conjugate-gradient sequence has stopped: inside an iteration the
// products and the cycle skip them. gmap: each row's graph (-1: never skipped), flag: per graph,
// nonzero once its sequence stopped; flag null: nothing is skipped.
struct RowSkip {
  const int32_t* gmap = nullptr;
  const int32_t* flag = nullptr;
};

__device__ __forceinline__ bool row_skipped(const RowSkip& k, int32_t row) {
  if (!k.flag) return false;
  const int32_t g = k.gmap[row];
  return g >= 0 && k.flag[g] != 0;
}

// m: row c of a block (6 values), x: the column's 6 values; V and X are float or double
template <typename V, typename X, typename A>
__device__ __forceinline__ A dot6(const V* __restrict__ m, const X* __restrict__ x) {
  using MV = typename Vec2<V>::T;
  using XV = typename Vec2<X>::T;
  const MV a = __ldg(reinterpret_cast<const MV*>(m)), b = __ldg(reinterpret_cast<const MV*>(m) + 1),
           d = __ldg(reinterpret_cast<const MV*>(m) + 2);
  const XV u = __ldg(reinterpret_cast<const XV*>(x)), v = __ldg(reinterpret_cast<const XV*>(x) + 1),
           w = __ldg(reinterpret_cast<const XV*>(x) + 2);
  return A(a.x) * A(u.x) + A(a.y) * A(u.y) + A(b.x) * A(v.x) + A(b.y) * A(v.y) + A(d.x) * A(w.x) + A(d.y) * A(w.y);
}

// (A x)_row,c in lanes c < 6 (other lanes: garbage); whole warp must call
template <typename V, typename X, typename A>
__device__ __forceinline__ A warp_row_product(int32_t k0, int32_t k1, const int32_t* __restrict__ col,
                                              const V* __restrict__ val, const X* __restrict__ x) {
  const int lane = threadIdx.x & 31;
  const int g = lane / 6, c = lane - 6 * (lane / 6);
  A acc = A(0);
  for (int32_t base = k0; base < k1; base += 30) {
    // up to 30 blocks: their columns in one load, then three passes of ten
    const int32_t nb = (k1 - base) < 30 ? (k1 - base) : 30;
    const int32_t mycol = lane < nb ? __ldg(col + base + lane) : 0;
    for (int32_t t = 0; t < nb; t += 10) {
      const int ia = t + g, ib = t + 5 + g;
      const int32_t ca = __shfl_sync(0xffffffffu, mycol, ia & 31);
      const int32_t cb = __shfl_sync(0xffffffffu, mycol, ib & 31);
      if (g < 5 && ia < nb) {
        const V* ma = val + 36 * int64_t(base + ia) + 6 * c;
        if (ib < nb) {
          const V* mb = val + 36 * int64_t(base + ib) + 6 * c;
          const A pa = dot6<V, X, A>(ma, x + 6 * int64_t(ca));
          const A pb = dot6<V, X, A>(mb, x + 6 * int64_t(cb));
          acc += pa + pb;
        } else {
          acc += dot6<V, X, A>(ma, x + 6 * int64_t(ca));
        }
      }
    }
  }
  const A a1 = __shfl_sync(0xffffffffu, acc, (c + 6) & 31);
  const A a2 = __shfl_sync(0xffffffffu, acc, (c + 12) & 31);
  const A a3 = __shfl_sync(0xffffffffu, acc, (c + 18) & 31);
  const A a4 = __shfl_sync(0xffffffffu, acc, (c + 24) & 31);
  return acc + a1 + a2 + a3 + a4;
}

// Schedules of the row product (chosen per operator by the table of sched_table.h, tune.cu; the
// two sum a row's blocks in different orders, so the choice is a fixed function of the operator's
// shape and never of a timing):
//   kWarpRow  one warp per block row, the five lane groups over the row's blocks (long rows)
//   kGroupRow five block rows per warp, one lane group per row, each lane over its row's blocks
//             (short rows: five rows in flight per warp)
enum Sched { kWarpRow = 0, kGroupRow = 1 };

template <int SCHED>
struct RowMap {
  static constexpr int kRowsPerWarp = SCHED == kWarpRow ? 1 : 5;
};

// The warp's rows: row of this lane's group (valid: row < n), component c of its output.
template <int SCHED>
__device__ __forceinline__ int32_t sched_row_of(int32_t warp, int* c_out, bool* lane_ok) {
  const int lane = threadIdx.x & 31;
  const int g = lane / 6;
  *c_out = lane - 6 * g;
  if (SCHED == kWarpRow) {
    *lane_ok = lane < 6;
    return warp;
  }
  *lane_ok = g < 5;
  return warp * 5 + (g < 5 ? g : 4);
}

// the block's warps take consecutive warp indices
template <int SCHED>
__device__ __forceinline__ int32_t sched_row(int rows_per_block_warps, int* c_out, bool* lane_ok) {
  return sched_row_of<SCHED>(int32_t(blockIdx.x) * rows_per_block_warps + (threadIdx.x >> 5), c_out, lane_ok);
}

// the row's product for this schedule; in kGroupRow every lane sums its own row's blocks
template <int SCHED, typename V, typename X, typename A>
__device__ __forceinline__ A sched_row_product(bool row_ok, int32_t row, const int32_t* __restrict__ rowptr,
                                               const int32_t* __restrict__ col, const V* __restrict__ val,
                                               const X* __restrict__ x) {
  if (SCHED == kWarpRow) {
    const int32_t k0 = row_ok ? rowptr[row] : 0, k1 = row_ok ? rowptr[row + 1] : 0;
    return warp_row_product<V, X, A>(k0, k1, col, val, x);
  }
  const int lane = threadIdx.x & 31;
  const int g = lane / 6, c = lane - 6 * g;
  A acc = A(0);
  if (row_ok && g < 5) {
    const int32_t k1 = rowptr[row + 1];
    int32_t k = rowptr[row];
    for (; k + 1 < k1; k += 2) {
      const int32_t ca = __ldg(col + k), cb = __ldg(col + k + 1);
      const A pa = dot6<V, X, A>(val + 36 * int64_t(k) + 6 * c, x + 6 * int64_t(ca));
      const A pb = dot6<V, X, A>(val + 36 * int64_t(k + 1) + 6 * c, x + 6 * int64_t(cb));
      acc += pa + pb;
    }
    if (k < k1) acc += dot6<V, X, A>(val + 36 * int64_t(k) + 6 * c, x + 6 * int64_t(__ldg(col + k)));
  }
  return acc;
}

// The slot schedule of the FP64 conjugate-gradient products. K's block rows are sorted by length
// once per K (solve.cu build_row_slots) into slots {row, first block, length}; lane group g (g < 5)
// of a warp takes R consecutive slots - rows of one length, as the sort puts them - and runs them
// in lock-step, lane 6g + c summing row c of each: per block step R column loads, then 3R value and
// 3R x loads, all independent, then 6R FMAs into R chains. The dependent chain per step is
// slot -> column -> x; lanes 30 and 31 idle. Six FMAs a block and row of output, the fewest the
// product can issue: GB300's FP64 rate bounds the FP64 product. (The FP32 products keep K's row
// order, whose neighbouring rows share value sectors and x in L1: sorted rows made the city block's
// FP32 CG product 41 -> 59-74 us.)
// SKIP: rows of stopped graphs (skip) come out not ok, with no product.
template <int R, typename V, typename X, typename A, bool SKIP = false>
__device__ __forceinline__ void slot_rows_product(const int4* __restrict__ slots, int64_t first, int64_t nslots,
                                                  const int32_t* __restrict__ col, const V* __restrict__ val,
                                                  const X* __restrict__ x, int32_t row[R], bool ok[R], A out[R],
                                                  RowSkip skip = RowSkip{}) {
  using MV = typename Vec2<V>::T;
  using XV = typename Vec2<X>::T;
  const int lane = threadIdx.x & 31;
  const int g = lane / 6, c = lane - 6 * g;
  int32_t k0[R], len[R];
  int32_t tmax = 0;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const int64_t sl = first + int64_t(g) * R + j;
    ok[j] = g < 5 && sl < nslots;
    int4 e = ok[j] ? __ldg(slots + sl) : make_int4(0, 0, 0, 0);
    if (SKIP && ok[j] && row_skipped(skip, e.x)) {
      ok[j] = false;
      e.z = 0;
    }
    row[j] = e.x;
    k0[j] = e.y;
    len[j] = e.z;
    tmax = len[j] > tmax ? len[j] : tmax;
    out[j] = A(0);
  }
  for (int32_t t = 0; t < tmax; ++t) {
    int32_t cl[R];
#pragma unroll
    for (int j = 0; j < R; ++j) cl[j] = t < len[j] ? __ldg(col + k0[j] + t) : 0;
    MV a[R][3];
    XV u[R][3];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (t < len[j]) {
        const MV* m = reinterpret_cast<const MV*>(val + 36 * int64_t(k0[j] + t) + 6 * c);
        const XV* v = reinterpret_cast<const XV*>(x + 6 * int64_t(cl[j]));
        a[j][0] = __ldg(m);
        a[j][1] = __ldg(m + 1);
        a[j][2] = __ldg(m + 2);
        u[j][0] = __ldg(v);
        u[j][1] = __ldg(v + 1);
        u[j][2] = __ldg(v + 2);
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (t < len[j]) {
        A acc = out[j];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          acc = fma(A(a[j][q].x), A(u[j][q].x), acc);
          acc = fma(A(a[j][q].y), A(u[j][q].y), acc);
        }
        out[j] = acc;
      }
    }
  }
}

// component q of the row's 6-vector v (held by the row's lanes) - whole warp must call
template <int SCHED, typename T>
__device__ __forceinline__ T row_component(T v, int q) {
  const int lane = threadIdx.x & 31;
  const int base = SCHED == kWarpRow ? 0 : 6 * ((lane / 6) < 5 ? lane / 6 : 4);
  return __shfl_sync(0xffffffffu, v, base + q);
}

}  // namespace svxg
