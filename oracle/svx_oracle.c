/* svx_oracle.c - TEST INFRASTRUCTURE ONLY: the oracle, a plain-C restatement of the reference's
 * stress solve (see svx_oracle.h). Every function names the reference lines it restates. Built
 * with -ffp-contract=off -fno-fast-math like the reference (CMakeLists.txt:17), so each
 * expression rounds exactly as the reference's does.
 */
#include "svx_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define ROW_GRAIN 512 /* kRowGrain, amg.hpp:31 */
#define DOT_GRAIN (8 * ROW_GRAIN) /* StressProblem::iterate's G, stress.cpp:407 */

/* std::max / std::min as the reference's <algorithm> evaluates them (NaN order included) */
#define MAXD(a, b) ((a) < (b) ? (b) : (a))
#define MIND(a, b) ((b) < (a) ? (b) : (a))

typedef struct { double x, y, z; } v3;

static v3 v3_of(svxg_v3 a) { v3 r = {a.x, a.y, a.z}; return r; }
static v3 v3_sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static double v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 v3_cross(v3 a, v3 b) {
  v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static double v3_at(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s);
  if (!p) abort();
  return p;
}
static void* xrealloc(void* p, size_t s) {
  void* q = realloc(p, s ? s : 1);
  if (!q) abort();
  return q;
}

/* ----------------------------------------------------------------------------------------------
 * 6x6 block kernels (amg.cpp:47-170, amg.hpp:132-161)
 * -------------------------------------------------------------------------------------------- */

/* blk6::inv6, amg.cpp:105-135: Gauss-Jordan with partial pivoting */
static int inv6(const double* A, double* Ainv) {
  double M[6][12];
  double scale = 0.0;
  for (int r = 0; r < 6; ++r) {
    for (int c = 0; c < 6; ++c) {
      M[r][c] = A[r * 6 + c];
      scale = MAXD(scale, fabs(M[r][c]));
    }
    for (int c = 0; c < 6; ++c) M[r][6 + c] = (r == c) ? 1.0 : 0.0;
  }
  if (scale == 0.0) return 0;
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    for (int r = c + 1; r < 6; ++r)
      if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
    if (fabs(M[piv][c]) <= 1e-15 * scale) return 0;
    if (piv != c)
      for (int k = 0; k < 12; ++k) {
        const double t = M[c][k];
        M[c][k] = M[piv][k];
        M[piv][k] = t;
      }
    const double inv = 1.0 / M[c][c];
    for (int k = 0; k < 12; ++k) M[c][k] *= inv;
    for (int r = 0; r < 6; ++r) {
      if (r == c) continue;
      const double f = M[r][c];
      if (f == 0.0) continue;
      for (int k = 0; k < 12; ++k) M[r][k] -= f * M[c][k];
    }
  }
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) Ainv[r * 6 + c] = M[r][6 + c];
  return 1;
}

/* blk6::fro6, amg.cpp:137-141 */
static double fro6(const double* M) {
  double s = 0.0;
  for (int i = 0; i < 36; ++i) s += M[i] * M[i];
  return sqrt(s);
}

/* blk6::rigid_block, amg.cpp:143-153: P = [[I, -[r]x], [0, I]] */
static void rigid_block(v3 r, double* P) {
  memset(P, 0, sizeof(double) * 36);
  for (int i = 0; i < 6; ++i) P[i * 6 + i] = 1.0;
  P[0 * 6 + 4] = r.z;
  P[0 * 6 + 5] = -r.y;
  P[1 * 6 + 3] = -r.z;
  P[1 * 6 + 5] = r.x;
  P[2 * 6 + 3] = r.y;
  P[2 * 6 + 4] = -r.x;
}

/* blk6::atbd_add, amg.cpp:155-170: T = B D, C += s A^T T */
static void atbd_add(const double* A, const double* B, const double* D, double s, double* C) {
  double T[36];
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) acc += B[r * 6 + k] * D[k * 6 + c];
      T[r * 6 + c] = acc;
    }
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) acc += A[k * 6 + r] * T[k * 6 + c];
      C[r * 6 + c] += s * acc;
    }
}

/* blk6::mv6 / mv6_add, amg.hpp:132-145 */
static void mv6(const double* M, const double* x, double* y) {
  const double x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3], x4 = x[4], x5 = x[5];
  for (int r = 0; r < 6; ++r) {
    const double* m = M + r * 6;
    y[r] = m[0] * x0 + m[1] * x1 + m[2] * x2 + m[3] * x3 + m[4] * x4 + m[5] * x5;
  }
}
static void mv6_add(const double* M, const double* x, double* y) {
  const double x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3], x4 = x[4], x5 = x[5];
  for (int r = 0; r < 6; ++r) {
    const double* m = M + r * 6;
    y[r] += m[0] * x0 + m[1] * x1 + m[2] * x2 + m[3] * x3 + m[4] * x4 + m[5] * x5;
  }
}

/* mul6, amg.cpp:59-67 (each element summed over q in order from zero) */
static void mul6(const double* A, const double* B, double* C) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int q = 0; q < 6; ++q) s += A[r * 6 + q] * B[q * 6 + c];
      C[r * 6 + c] = s;
    }
}
/* mul6_add<trans>, amg.cpp:69-78: C += A B (A^T B if trans) */
static void mul6_add(int trans, const double* A, const double* B, double* C) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int q = 0; q < 6; ++q) s += (trans ? A[q * 6 + r] : A[r * 6 + q]) * B[q * 6 + c];
      C[r * 6 + c] = C[r * 6 + c] + s;
    }
}

/* bsub / badd, amg.cpp:80-93: (y0, y1) -/+= B x, B column-major padded to 8 rows */
static void bsub(const float* B, const float* x, float* y) {
  for (int j = 0; j < 6; ++j) {
    const float xj = x[j];
    for (int r = 0; r < 8; ++r) y[r] -= B[8 * j + r] * xj;
  }
}
static void badd(const float* B, const float* x, float* y) {
  for (int j = 0; j < 6; ++j) {
    const float xj = x[j];
    for (int r = 0; r < 8; ++r) y[r] += B[8 * j + r] * xj;
  }
}
/* to_f32_block, amg.cpp:94-99 */
static void to_f32_block(const double* B, float* out) {
  for (int c = 0; c < 6; ++c) {
    for (int r = 0; r < 6; ++r) out[8 * c + r] = (float)B[r * 6 + c];
    out[8 * c + 6] = out[8 * c + 7] = 0.0f;
  }
}

/* ----------------------------------------------------------------------------------------------
 * Bsr6 and its builder (amg.cpp:174-224)
 * -------------------------------------------------------------------------------------------- */

typedef struct {
  int32_t n;
  int64_t nnzb;
  int32_t* rowptr;
  int32_t* col;
  double* val;
} bsr;

static void bsr_free(bsr* A) {
  free(A->rowptr);
  free(A->col);
  free(A->val);
  memset(A, 0, sizeof(*A));
}

static bsr bsr_copy(const bsr* A) {
  bsr B = *A;
  B.rowptr = xcalloc((size_t)A->n + 1, sizeof(int32_t));
  B.col = xcalloc((size_t)A->nnzb, sizeof(int32_t));
  B.val = xcalloc((size_t)A->nnzb * 36, sizeof(double));
  memcpy(B.rowptr, A->rowptr, sizeof(int32_t) * ((size_t)A->n + 1));
  memcpy(B.col, A->col, sizeof(int32_t) * (size_t)A->nnzb);
  memcpy(B.val, A->val, sizeof(double) * 36 * (size_t)A->nnzb);
  return B;
}

/* Bsr6::apply, amg.cpp:174-183 (rows in 512-row chunks) */
static void bsr_apply(const bsr* A, const double* x, double* y) {
  const int64_t nch = ((int64_t)A->n + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel for schedule(static)
  for (int64_t ch = 0; ch < nch; ++ch) {
    const int64_t r1 = MIND((int64_t)A->n, (ch + 1) * ROW_GRAIN);
    for (int64_t i = ch * ROW_GRAIN; i < r1; ++i) {
      double* yi = y + 6 * i;
      for (int q = 0; q < 6; ++q) yi[q] = 0.0;
      for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1]; ++k)
        mv6_add(&A->val[36 * (size_t)k], x + 6 * (size_t)A->col[k], yi);
    }
  }
}

/* Bsr6Builder, amg.cpp:185-224: per row (col, slot) pairs in first-use order, blocks
 * zero-initialised on first use; finish(): diagonal first, then ascending columns. */
typedef struct {
  int32_t cnt, cap;
  int32_t* col;
  int32_t* slot;
} brow;
typedef struct {
  int32_t n;
  brow* rows;
  double* store;
  int64_t nslots, cap;
} builder;

static void builder_init(builder* B, int32_t n) {
  B->n = n;
  B->rows = xcalloc((size_t)n, sizeof(brow));
  B->store = NULL;
  B->nslots = B->cap = 0;
}

static double* builder_block(builder* B, int32_t r, int32_t c) {
  brow* row = &B->rows[r];
  for (int32_t e = 0; e < row->cnt; ++e)
    if (row->col[e] == c) return &B->store[36 * (size_t)row->slot[e]];
  if (B->nslots == B->cap) {
    B->cap = B->cap ? 2 * B->cap : 1024;
    B->store = xrealloc(B->store, sizeof(double) * 36 * (size_t)B->cap);
  }
  const int64_t slot = B->nslots++;
  memset(&B->store[36 * (size_t)slot], 0, sizeof(double) * 36);
  if (row->cnt == row->cap) {
    row->cap = row->cap ? 2 * row->cap : 8;
    row->col = xrealloc(row->col, sizeof(int32_t) * (size_t)row->cap);
    row->slot = xrealloc(row->slot, sizeof(int32_t) * (size_t)row->cap);
  }
  row->col[row->cnt] = c;
  row->slot[row->cnt] = (int32_t)slot;
  row->cnt++;
  return &B->store[36 * (size_t)slot];
}

static bsr builder_finish(builder* B) {
  bsr A;
  A.n = B->n;
  A.rowptr = xcalloc((size_t)B->n + 1, sizeof(int32_t));
  int64_t nnz = 0;
  for (int32_t r = 0; r < B->n; ++r) {
    brow* row = &B->rows[r];
    /* insertion sort: the diagonal first, then ascending columns (columns are unique) */
    for (int32_t a = 1; a < row->cnt; ++a) {
      const int32_t c = row->col[a], s = row->slot[a];
      int32_t b = a - 1;
      while (b >= 0) {
        const int32_t cb = row->col[b];
        const int before = (c == r) ? (cb != r) : (cb != r && c < cb);
        if (!before) break;
        row->col[b + 1] = row->col[b];
        row->slot[b + 1] = row->slot[b];
        --b;
      }
      row->col[b + 1] = c;
      row->slot[b + 1] = s;
    }
    int has_diag = row->cnt > 0 && row->col[0] == r;
    nnz += row->cnt + (has_diag ? 0 : 1);
    A.rowptr[r + 1] = (int32_t)nnz;
  }
  A.nnzb = nnz;
  A.col = xcalloc((size_t)nnz, sizeof(int32_t));
  A.val = xcalloc((size_t)nnz * 36, sizeof(double));
  int64_t k = 0;
  for (int32_t r = 0; r < B->n; ++r) {
    brow* row = &B->rows[r];
    if (!(row->cnt > 0 && row->col[0] == r)) A.col[k++] = r; /* (an empty diagonal) */
    for (int32_t e = 0; e < row->cnt; ++e) {
      A.col[k] = row->col[e];
      memcpy(&A.val[36 * (size_t)k], &B->store[36 * (size_t)row->slot[e]], sizeof(double) * 36);
      ++k;
    }
    free(row->col);
    free(row->slot);
  }
  free(B->rows);
  free(B->store);
  memset(B, 0, sizeof(*B));
  return A;
}

/* ----------------------------------------------------------------------------------------------
 * The multigrid (amg.hpp:71-118, amg.cpp:228-731)
 * -------------------------------------------------------------------------------------------- */

typedef struct {
  bsr A;
  double* Dinv;
  v3* pos;
  int32_t* parent;
  v3* off;
  int32_t *Prow, *Pcol;
  double* Pval;
  int64_t pnnz;
  double lmax;
  int32_t* Rrow;
  int32_t *Rent_i, *Rent_e;
  int32_t nc; /* the next level's size (restriction rows) */
  float *Af, *Df, *Pf, *Rf;
  float *xf, *bf, *rf, *of, *cf;
} level;

typedef struct {
  svxg_amg_options opt;
  int32_t nlev;
  level lv[16];
  double* chol;
  int32_t chol_n;
  int64_t work, build_work;
  int keep; /* keep the double-precision copies (hierarchy export) */
} amg;

static void level_free(level* L) {
  bsr_free(&L->A);
  free(L->Dinv);
  free(L->pos);
  free(L->parent);
  free(L->off);
  free(L->Prow);
  free(L->Pcol);
  free(L->Pval);
  free(L->Rrow);
  free(L->Rent_i);
  free(L->Rent_e);
  free(L->Af);
  free(L->Df);
  free(L->Pf);
  free(L->Rf);
  free(L->xf);
  free(L->bf);
  free(L->rf);
  free(L->of);
  free(L->cf);
  memset(L, 0, sizeof(*L));
}

static void amg_clear(amg* M) {
  for (int32_t l = 0; l < M->nlev; ++l) level_free(&M->lv[l]);
  M->nlev = 0;
  free(M->chol);
  M->chol = NULL;
  M->chol_n = 0;
  M->work = M->build_work = 0;
}

static double estimate_lmax(amg* M, const level* L);

/* Amg::finalize, amg.cpp:228-254 */
static int finalize(amg* M, level* L) {
  const int32_t n = L->A.n;
  L->Dinv = xcalloc(36 * (size_t)n, sizeof(double));
  for (int32_t i = 0; i < n; ++i) {
    const double* D = &L->A.val[36 * (size_t)L->A.rowptr[i]];
    if (!inv6(D, &L->Dinv[36 * (size_t)i])) {
      double Dr[36];
      memcpy(Dr, D, sizeof(Dr));
      double tr = 0.0;
      for (int q = 0; q < 6; ++q) tr += fabs(Dr[q * 7]);
      const double eps = tr > 0 ? 1e-9 * tr : 1.0;
      for (int q = 0; q < 6; ++q) Dr[q * 7] += eps;
      if (!inv6(Dr, &L->Dinv[36 * (size_t)i])) return 0;
    }
  }
  M->build_work += 12 * (int64_t)n;
  if (!M->opt.sgs) L->lmax = estimate_lmax(M, L);
  return 1;
}

/* Amg::estimate_lmax, amg.cpp:256-275: power iteration on D^-1 A */
static double estimate_lmax(amg* M, const level* L) {
  const int32_t n = L->A.n;
  M->build_work += 15 * (L->A.nnzb + n);
  const size_t m = 6 * (size_t)n;
  double* v = xcalloc(m, sizeof(double));
  double* w = xcalloc(m, sizeof(double));
  for (size_t k = 0; k < m; ++k) v[k] = 1.0 + 0.001 * (double)(k % 7);
  double lam = 1.0;
  for (int it = 0; it < 15; ++it) {
    bsr_apply(&L->A, v, w);
    for (int32_t i = 0; i < n; ++i) mv6(&L->Dinv[36 * (size_t)i], &w[6 * (size_t)i], &v[6 * (size_t)i]);
    double nv = 0.0;
    for (size_t k = 0; k < m; ++k) nv += v[k] * v[k];
    nv = sqrt(nv);
    if (!(nv > 0)) break;
    lam = nv;
    for (size_t k = 0; k < m; ++k) v[k] /= nv;
  }
  free(v);
  free(w);
  return 1.1 * lam;
}

/* per-row sparse accumulator entries of the prolongation and Galerkin products */
typedef struct {
  int32_t cnt, cap;
  int32_t* c;
  double* b; /* 36 per entry */
} acc_row;

static double* acc_slot(acc_row* row, int32_t* slot, int32_t c) {
  int32_t at = slot[c];
  if (at < 0) {
    if (row->cnt == row->cap) {
      row->cap = row->cap ? 2 * row->cap : 8;
      row->c = xrealloc(row->c, sizeof(int32_t) * (size_t)row->cap);
      row->b = xrealloc(row->b, sizeof(double) * 36 * (size_t)row->cap);
    }
    at = row->cnt++;
    slot[c] = at;
    row->c[at] = c;
    memset(&row->b[36 * (size_t)at], 0, sizeof(double) * 36);
  }
  return &row->b[36 * (size_t)at];
}

/* Amg::coarsen, amg.cpp:320-533. Appends level l + 1; 0 if coarsening does not pay. */
/* Pass 3's grouping of uncoupled leftover rows (the reference's, on); off only for checking the
   library's batches of graphs, whose multigrid keeps such rows single (svxo_set_group_isolated). */
static int g_group_isolated = 1;
void svxo_set_group_isolated(int on) { g_group_isolated = on != 0; }

static int coarsen(amg* M, int32_t l, int smoothed) {
  level* F = &M->lv[l];
  const bsr* A = &F->A;
  const int32_t n = A->n;
  double* dn = xcalloc((size_t)n, sizeof(double));
  for (int32_t i = 0; i < n; ++i) dn[i] = fro6(&A->val[36 * (size_t)A->rowptr[i]]);
  double theta = M->opt.strength;
  int32_t* agg = xcalloc((size_t)n, sizeof(int32_t));
  int32_t* agg1 = xcalloc((size_t)n, sizeof(int32_t));
  int32_t na = 0;
#define ISOLATED(i) (A->rowptr[(i) + 1] - A->rowptr[(i)] <= 1)
#define STRONG(i, k)                                                                                             \
  (A->col[k] != (i) &&                                                                                           \
   fro6(&A->val[36 * (size_t)(k)]) >= theta * sqrt(dn[(i)] * dn[A->col[k]]))
  for (int round = 0;; ++round) {
    for (int32_t i = 0; i < n; ++i) agg[i] = -1;
    na = 0;
    /* pass 1: roots whose strong neighbourhood is free */
    for (int32_t i = 0; i < n; ++i) {
      if (agg[i] >= 0 || ISOLATED(i)) continue;
      int isfree = 1;
      for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1] && isfree; ++k)
        if (STRONG(i, k) && agg[A->col[k]] >= 0) isfree = 0;
      if (!isfree) continue;
      agg[i] = na;
      for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1]; ++k)
        if (STRONG(i, k)) agg[A->col[k]] = na;
      ++na;
    }
    /* pass 2: join the most strongly coupled aggregated neighbour */
    memcpy(agg1, agg, sizeof(int32_t) * (size_t)n);
    for (int32_t i = 0; i < n; ++i) {
      if (agg1[i] >= 0) continue;
      double best = -1.0;
      int32_t ba = -1;
      for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1]; ++k) {
        const int32_t j = A->col[k];
        if (j == i || agg1[j] < 0) continue;
        const double s = fro6(&A->val[36 * (size_t)k]);
        if (s > best) {
          best = s;
          ba = agg1[j];
        }
      }
      agg[i] = ba;
    }
    /* pass 3: leftovers; uncoupled rows grouped eight at a time (each its own with
       g_group_isolated off: the batch form of the library, whose graphs must stay apart) */
    {
      int32_t open = -1, fill = 0;
      for (int32_t i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        if (!ISOLATED(i) || !g_group_isolated) {
          agg[i] = na++;
          continue;
        }
        if (open < 0 || fill >= 8) {
          open = na++;
          fill = 0;
        }
        agg[i] = open;
        ++fill;
      }
    }
    if (!M->opt.reaggregate || round == 3 || 2 * (int64_t)na <= n) break;
    theta *= 0.5;
  }
#undef STRONG
  free(agg1);
  free(dn);
  if (na >= n || (double)na > 0.85 * n) {
    free(agg);
    return 0;
  }
  level* C = &M->lv[l + 1];
  memset(C, 0, sizeof(*C));
  C->pos = xcalloc((size_t)na, sizeof(v3));
  int32_t* cnt = xcalloc((size_t)na, sizeof(int32_t));
  for (int32_t i = 0; i < n; ++i) {
    v3* p = &C->pos[agg[i]];
    p->x += F->pos[i].x;
    p->y += F->pos[i].y;
    p->z += F->pos[i].z;
    ++cnt[agg[i]];
  }
  for (int32_t a = 0; a < na; ++a) {
    const double s = 1.0 / cnt[a];
    C->pos[a].x *= s;
    C->pos[a].y *= s;
    C->pos[a].z *= s;
  }
  free(cnt);
  F->parent = agg;
  F->off = xcalloc((size_t)n, sizeof(v3));
  for (int32_t i = 0; i < n; ++i) F->off[i] = v3_sub(F->pos[i], C->pos[agg[i]]);
  /* prolongation: rigid modes of each aggregate, smoothed by one damped Jacobi step */
  {
    acc_row* rows = xcalloc((size_t)n, sizeof(acc_row));
    const double lmax = smoothed ? estimate_lmax(M, F) : 0.0;
    const double omega = smoothed ? (4.0 / 3.0) / MAXD(1e-300, lmax) : 0.0;
    const int64_t nch = ((int64_t)n + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel
    {
      int32_t* slot = xcalloc((size_t)na, sizeof(int32_t));
      for (int32_t a = 0; a < na; ++a) slot[a] = -1;
#pragma omp for schedule(static)
      for (int64_t ch = 0; ch < nch; ++ch) {
        const int64_t i1 = MIND((int64_t)n, (ch + 1) * ROW_GRAIN);
        for (int64_t i = ch * ROW_GRAIN; i < i1; ++i) {
          acc_row* row = &rows[i];
          double Pt[36];
          rigid_block(F->off[i], Pt);
          double* b = acc_slot(row, slot, agg[i]);
          for (int q = 0; q < 36; ++q) b[q] += 1.0 * Pt[q];
          const double* Di = &F->Dinv[36 * (size_t)i];
          const int32_t kend = omega != 0.0 ? A->rowptr[i + 1] : A->rowptr[i];
          for (int32_t k = A->rowptr[i]; k < kend; ++k) {
            const int32_t j = A->col[k];
            double Pj[36], T[36], U[36];
            rigid_block(F->off[j], Pj);
            mul6(&A->val[36 * (size_t)k], Pj, T);
            mul6(Di, T, U);
            double* bj = acc_slot(row, slot, agg[j]);
            for (int q = 0; q < 36; ++q) bj[q] += -omega * U[q];
          }
          for (int32_t e = 0; e < row->cnt; ++e) slot[row->c[e]] = -1;
        }
      }
      free(slot);
    }
    F->Prow = xcalloc((size_t)n + 1, sizeof(int32_t));
    int64_t total = 0;
    for (int32_t i = 0; i < n; ++i) total += rows[i].cnt;
    F->Pcol = xcalloc((size_t)total, sizeof(int32_t));
    F->Pval = xcalloc((size_t)total * 36, sizeof(double));
    F->pnnz = total;
    int64_t e0 = 0;
    for (int32_t i = 0; i < n; ++i) {
      acc_row* row = &rows[i];
      /* sort by coarse column (insertion sort: rows are short, columns unique) */
      int32_t* ord = xcalloc((size_t)row->cnt, sizeof(int32_t));
      for (int32_t e = 0; e < row->cnt; ++e) ord[e] = e;
      for (int32_t a = 1; a < row->cnt; ++a) {
        const int32_t t = ord[a];
        int32_t b = a - 1;
        while (b >= 0 && row->c[ord[b]] > row->c[t]) {
          ord[b + 1] = ord[b];
          --b;
        }
        ord[b + 1] = t;
      }
      for (int32_t e = 0; e < row->cnt; ++e) {
        F->Pcol[e0] = row->c[ord[e]];
        memcpy(&F->Pval[36 * (size_t)e0], &row->b[36 * (size_t)ord[e]], sizeof(double) * 36);
        ++e0;
      }
      F->Prow[i + 1] = (int32_t)e0;
      free(ord);
      free(row->c);
      free(row->b);
    }
    free(rows);
  }
  if (smoothed) M->build_work += 12 * A->nnzb;
  for (int32_t i = 0; i < n; ++i)
    for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1]; ++k) {
      const int32_t j = A->col[k];
      M->build_work += 6 * (int64_t)(F->Prow[j + 1] - F->Prow[j]);
    }
  /* restriction lists: P^T by coarse node */
  F->nc = na;
  F->Rrow = xcalloc((size_t)na + 1, sizeof(int32_t));
  for (int64_t e = 0; e < F->pnnz; ++e) ++F->Rrow[F->Pcol[e] + 1];
  for (int32_t a = 0; a < na; ++a) F->Rrow[a + 1] += F->Rrow[a];
  F->Rent_i = xcalloc((size_t)F->pnnz, sizeof(int32_t));
  F->Rent_e = xcalloc((size_t)F->pnnz, sizeof(int32_t));
  {
    int32_t* fill = xcalloc((size_t)na, sizeof(int32_t));
    memcpy(fill, F->Rrow, sizeof(int32_t) * (size_t)na);
    for (int32_t i = 0; i < n; ++i)
      for (int32_t e = F->Prow[i]; e < F->Prow[i + 1]; ++e) {
        const int32_t at = fill[F->Pcol[e]]++;
        F->Rent_i[at] = i;
        F->Rent_e[at] = e;
      }
    free(fill);
  }
  /* Galerkin product A_c = P^T (A P): A P by fine row, then P^T (A P) by coarse row */
  acc_row* apr = xcalloc((size_t)n, sizeof(acc_row));
  {
    const int64_t nch = ((int64_t)n + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel
    {
      int32_t* slot = xcalloc((size_t)na, sizeof(int32_t));
      for (int32_t a = 0; a < na; ++a) slot[a] = -1;
#pragma omp for schedule(static)
      for (int64_t ch = 0; ch < nch; ++ch) {
        const int64_t i1 = MIND((int64_t)n, (ch + 1) * ROW_GRAIN);
        for (int64_t i = ch * ROW_GRAIN; i < i1; ++i) {
          acc_row* ap = &apr[i];
          for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1]; ++k) {
            const int32_t j = A->col[k];
            const double* Aij = &A->val[36 * (size_t)k];
            for (int32_t e = F->Prow[j]; e < F->Prow[j + 1]; ++e) {
              double* dst = acc_slot(ap, slot, F->Pcol[e]);
              mul6_add(0, Aij, &F->Pval[36 * (size_t)e], dst);
            }
          }
          for (int32_t e = 0; e < ap->cnt; ++e) slot[ap->c[e]] = -1;
        }
      }
      free(slot);
    }
  }
  for (int32_t i = 0; i < n; ++i) M->build_work += 6 * (int64_t)(F->Prow[i + 1] - F->Prow[i]) * (int64_t)apr[i].cnt;
  acc_row* crow = xcalloc((size_t)na, sizeof(acc_row));
  {
    const int64_t nch = ((int64_t)na + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel
    {
      int32_t* slot = xcalloc((size_t)na, sizeof(int32_t));
      for (int32_t a = 0; a < na; ++a) slot[a] = -1;
#pragma omp for schedule(static)
      for (int64_t ch = 0; ch < nch; ++ch) {
        const int64_t a1 = MIND((int64_t)na, (ch + 1) * ROW_GRAIN);
        for (int64_t I = ch * ROW_GRAIN; I < a1; ++I) {
          acc_row* out = &crow[I];
          for (int32_t r = F->Rrow[I]; r < F->Rrow[I + 1]; ++r) {
            const int32_t i = F->Rent_i[r], e = F->Rent_e[r];
            const double* Pi = &F->Pval[36 * (size_t)e];
            const acc_row* x = &apr[i];
            for (int32_t t = 0; t < x->cnt; ++t) {
              double* dst = acc_slot(out, slot, x->c[t]);
              mul6_add(1, Pi, &x->b[36 * (size_t)t], dst);
            }
          }
          for (int32_t t = 0; t < out->cnt; ++t) slot[out->c[t]] = -1;
        }
      }
      free(slot);
    }
  }
  for (int32_t i = 0; i < n; ++i) {
    free(apr[i].c);
    free(apr[i].b);
  }
  free(apr);
  builder B;
  builder_init(&B, na);
  for (int32_t I = 0; I < na; ++I) {
    for (int32_t t = 0; t < crow[I].cnt; ++t) {
      double* dst = builder_block(&B, I, crow[I].c[t]);
      for (int q = 0; q < 36; ++q) dst[q] += crow[I].b[36 * (size_t)t + q];
    }
    free(crow[I].c);
    free(crow[I].b);
  }
  free(crow);
  C->A = builder_finish(&B);
  if (!smoothed && M->opt.coarse_scale != 1.0)
    for (int64_t q = 0; q < 36 * C->A.nnzb; ++q) C->A.val[q] *= M->opt.coarse_scale;
  if (!finalize(M, C)) {
    level_free(C);
    return 0;
  }
  M->nlev = l + 2;
  return 1;
}

/* Amg::factor_coarsest, amg.cpp:535-578 */
static void factor_coarsest(amg* M) {
  const level* L = &M->lv[M->nlev - 1];
  if (L->A.n > 4 * M->opt.coarse_max) {
    M->chol_n = 0;
    free(M->chol);
    M->chol = NULL;
    return;
  }
  const int32_t m = 6 * L->A.n;
  M->chol_n = m;
  M->build_work += (int64_t)m * m * m / 108;
  free(M->chol);
  double* C = M->chol = xcalloc((size_t)m * (size_t)m, sizeof(double));
  for (int32_t i = 0; i < L->A.n; ++i)
    for (int32_t k = L->A.rowptr[i]; k < L->A.rowptr[i + 1]; ++k) {
      const int32_t j = L->A.col[k];
      const double* b = &L->A.val[36 * (size_t)k];
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) C[(size_t)(6 * i + r) * m + (size_t)(6 * j + c)] += b[r * 6 + c];
    }
  double dmax = 0.0;
  for (int32_t i = 0; i < m; ++i) dmax = MAXD(dmax, fabs(C[(size_t)i * m + i]));
  for (int32_t j = 0; j < m; ++j) {
    double d = C[(size_t)j * m + j];
    for (int32_t k = 0; k < j; ++k) d -= C[(size_t)j * m + k] * C[(size_t)j * m + k];
    if (!(d > 1e-12 * dmax)) d = MAXD(1e-12 * dmax, 1e-300);
    const double s = sqrt(d);
    C[(size_t)j * m + j] = s;
#pragma omp parallel for schedule(static)
    for (int32_t i = j + 1; i < m; ++i) {
      double v = 0.5 * (C[(size_t)i * m + j] + C[(size_t)j * m + i]);
      for (int32_t k = 0; k < j; ++k) v -= C[(size_t)i * m + k] * C[(size_t)j * m + k];
      C[(size_t)i * m + j] = v / s;
    }
  }
  for (int32_t i = 0; i < m; ++i)
    for (int32_t k = i + 1; k < m; ++k) C[(size_t)i * m + k] = C[(size_t)k * m + i];
}

/* Amg::solve_coarsest, amg.cpp:580-592 */
static void solve_coarsest(const amg* M, const double* b, double* x) {
  const int32_t m = M->chol_n;
  const double* C = M->chol;
  for (int32_t i = 0; i < m; ++i) {
    double v = b[i];
    for (int32_t k = 0; k < i; ++k) v -= C[(size_t)i * m + k] * x[k];
    x[i] = v / C[(size_t)i * m + i];
  }
  for (int32_t i = m - 1; i >= 0; --i) {
    double v = x[i];
    for (int32_t k = i + 1; k < m; ++k) v -= C[(size_t)i * m + k] * x[k];
    x[i] = v / C[(size_t)i * m + i];
  }
}

/* Amg::make_fast, amg.cpp:594-628 (double-precision copies kept when exporting) */
static void make_fast(amg* M) {
  for (int32_t l = 0; l < M->nlev; ++l) {
    level* L = &M->lv[l];
    const size_t nb = (size_t)L->A.nnzb;
    L->Af = xcalloc(48 * nb, sizeof(float));
    for (size_t k = 0; k < nb; ++k) to_f32_block(&L->A.val[36 * k], &L->Af[48 * k]);
    L->Df = xcalloc(48 * (size_t)L->A.n, sizeof(float));
    for (int32_t i = 0; i < L->A.n; ++i) to_f32_block(&L->Dinv[36 * (size_t)i], &L->Df[48 * (size_t)i]);
    L->Pf = xcalloc(48 * (size_t)L->pnnz, sizeof(float));
    for (int64_t e = 0; e < L->pnnz; ++e) to_f32_block(&L->Pval[36 * (size_t)e], &L->Pf[48 * (size_t)e]);
    L->Rf = xcalloc(48 * (size_t)L->pnnz, sizeof(float));
    for (int64_t r = 0; r < L->pnnz; ++r) {
      const double* P = &L->Pval[36 * (size_t)L->Rent_e[r]];
      double T[36];
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 6; ++b) T[a * 6 + b] = P[b * 6 + a];
      to_f32_block(T, &L->Rf[48 * (size_t)r]);
    }
    const size_t m = 8 * (size_t)L->A.n;
    L->xf = xcalloc(m, sizeof(float));
    L->bf = xcalloc(m, sizeof(float));
    L->rf = xcalloc(m, sizeof(float));
    L->of = xcalloc(m, sizeof(float));
    L->cf = xcalloc(m, sizeof(float));
  }
}

/* Amg::build, amg.cpp:277-318 */
static int amg_build(amg* M, const bsr* A, const v3* pos, const svxg_amg_options* opt) {
  const int keep = M->keep;
  amg_clear(M);
  M->keep = keep;
  M->opt = *opt;
  if (A->n == 0) return 1;
  M->nlev = 1;
  memset(&M->lv[0], 0, sizeof(level));
  M->lv[0].A = bsr_copy(A);
  M->lv[0].pos = xcalloc((size_t)A->n, sizeof(v3));
  memcpy(M->lv[0].pos, pos, sizeof(v3) * (size_t)A->n);
  if (!finalize(M, &M->lv[0])) {
    amg_clear(M);
    return 0;
  }
  while (M->nlev < M->opt.max_levels && M->nlev < 16 && M->lv[M->nlev - 1].A.n > M->opt.coarse_max) {
    const bsr* L = &M->lv[M->nlev - 1].A;
    const int dense = M->nlev > 1 && L->nnzb > 80 * (int64_t)L->n;
    if (dense && !M->opt.coarsen_dense) break;
    if (!coarsen(M, M->nlev - 1, !dense && M->opt.smoothed)) break;
    if (dense) break;
  }
  factor_coarsest(M);
  make_fast(M);
  for (int32_t l = 0; l < M->nlev; ++l) {
    const int last = l + 1 == M->nlev;
    const int64_t nd = M->opt.dense_work_per_unknown ? M->chol_n : M->chol_n / 6;
    const int64_t blocks = M->lv[l].A.nnzb;
    const int64_t coarsest = M->chol_n > 0 ? MAXD(blocks, 2 * nd * nd) : 8 * 2 * blocks;
    const int64_t per = last ? coarsest : blocks * (4 * M->opt.sweeps + 2);
    int64_t g = 1;
    for (int32_t k = 0; k < l; ++k) g *= M->opt.gamma;
    M->work += per * g;
  }
  return 1;
}

/* Amg::smooth_f, amg.cpp:630-659: hybrid Gauss-Seidel over fixed 512-row blocks */
static void smooth_f(const level* L, float* x, const float* b, int fresh, int backward) {
  const bsr* A = &L->A;
  const int32_t n = A->n;
  if (!fresh) memcpy(L->of, x, sizeof(float) * 8 * (size_t)n);
  const float* xo = L->of;
  const int64_t nch = ((int64_t)n + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel for schedule(static)
  for (int64_t ch = 0; ch < nch; ++ch) {
    const int64_t r0 = ch * ROW_GRAIN, r1 = MIND((int64_t)n, (ch + 1) * ROW_GRAIN);
    for (int64_t ii = 0; ii < r1 - r0; ++ii) {
      const int64_t i = backward ? r1 - 1 - ii : r0 + ii;
      float s[8], y[8];
      for (int q = 0; q < 8; ++q) s[q] = b[8 * i + q];
      const int32_t k1 = A->rowptr[i + 1];
      for (int32_t k = A->rowptr[i] + 1; k < k1; ++k) {
        const int64_t j = A->col[k];
        if (j >= r0 && j < r1) {
          if (fresh && j > i) continue;
          bsub(&L->Af[48 * (size_t)k], x + 8 * j, s);
        } else if (!fresh) {
          bsub(&L->Af[48 * (size_t)k], xo + 8 * j, s);
        }
      }
      for (int q = 0; q < 8; ++q) y[q] = 0.0f;
      badd(&L->Df[48 * (size_t)i], s, y);
      for (int q = 0; q < 8; ++q) x[8 * i + q] = y[q];
    }
  }
}

/* Amg::cycle_f, amg.cpp:661-716 */
static void cycle_f(const amg* M, int32_t l, const float* b, float* x) {
  const level* L = &M->lv[l];
  const int32_t n = L->A.n;
  if (l + 1 == M->nlev && M->chol_n == 0) {
    for (int sw = 0; sw < 4; ++sw) smooth_f(L, x, b, sw == 0, 0);
    for (int sw = 0; sw < 4; ++sw) smooth_f(L, x, b, 0, 1);
    return;
  }
  if (l + 1 == M->nlev) {
    double* bd = xcalloc(6 * (size_t)n, sizeof(double));
    double* xd = xcalloc(6 * (size_t)n, sizeof(double));
    for (int32_t i = 0; i < n; ++i)
      for (int q = 0; q < 6; ++q) bd[6 * (size_t)i + q] = b[8 * (size_t)i + q];
    solve_coarsest(M, bd, xd);
    for (int32_t i = 0; i < n; ++i) {
      for (int q = 0; q < 6; ++q) x[8 * (size_t)i + q] = (float)xd[6 * (size_t)i + q];
      x[8 * (size_t)i + 6] = x[8 * (size_t)i + 7] = 0.0f;
    }
    free(bd);
    free(xd);
    return;
  }
  for (int sw = 0; sw < M->opt.sweeps; ++sw) smooth_f(L, x, b, sw == 0, 0);
  const bsr* A = &L->A;
  float* r = L->rf;
  {
    const int64_t nch = ((int64_t)n + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel for schedule(static)
    for (int64_t ch = 0; ch < nch; ++ch) {
      const int64_t r1 = MIND((int64_t)n, (ch + 1) * ROW_GRAIN);
      for (int64_t i = ch * ROW_GRAIN; i < r1; ++i) {
        float s[8];
        for (int q = 0; q < 8; ++q) s[q] = b[8 * i + q];
        for (int32_t k = A->rowptr[i]; k < A->rowptr[i + 1]; ++k)
          bsub(&L->Af[48 * (size_t)k], x + 8 * (size_t)A->col[k], s);
        for (int q = 0; q < 8; ++q) r[8 * i + q] = s[q];
      }
    }
  }
  const level* C = &M->lv[l + 1];
  float* bc = C->bf;
  {
    const int64_t nc = C->A.n;
    const int64_t nch = (nc + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel for schedule(static)
    for (int64_t ch = 0; ch < nch; ++ch) {
      const int64_t a1 = MIND(nc, (ch + 1) * ROW_GRAIN);
      for (int64_t a = ch * ROW_GRAIN; a < a1; ++a) {
        float y[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int32_t e = L->Rrow[a]; e < L->Rrow[a + 1]; ++e)
          badd(&L->Rf[48 * (size_t)e], r + 8 * (size_t)L->Rent_i[e], y);
        for (int q = 0; q < 8; ++q) bc[8 * a + q] = y[q];
      }
    }
  }
  float* xc = L->cf;
  cycle_f(M, l + 1, bc, xc);
  {
    const int64_t nch = ((int64_t)n + ROW_GRAIN - 1) / ROW_GRAIN;
#pragma omp parallel for schedule(static)
    for (int64_t ch = 0; ch < nch; ++ch) {
      const int64_t r1 = MIND((int64_t)n, (ch + 1) * ROW_GRAIN);
      for (int64_t i = ch * ROW_GRAIN; i < r1; ++i) {
        float y[8];
        for (int q = 0; q < 8; ++q) y[q] = x[8 * i + q];
        for (int32_t e = L->Prow[i]; e < L->Prow[i + 1]; ++e)
          badd(&L->Pf[48 * (size_t)e], xc + 8 * (size_t)L->Pcol[e], y);
        for (int q = 0; q < 8; ++q) x[8 * i + q] = y[q];
      }
    }
  }
  for (int sw = 0; sw < M->opt.sweeps; ++sw) smooth_f(L, x, b, 0, 1);
}

/* Amg::apply, amg.cpp:718-731 */
static void amg_apply(const amg* M, const double* r, double* z) {
  if (M->nlev == 0) return;
  const level* L = &M->lv[0];
  const int32_t n = L->A.n;
  float* b = L->bf;
  for (int32_t i = 0; i < n; ++i) {
    for (int q = 0; q < 6; ++q) b[8 * (size_t)i + q] = (float)r[6 * (size_t)i + q];
    b[8 * (size_t)i + 6] = b[8 * (size_t)i + 7] = 0.0f;
  }
  float* x = L->xf;
  cycle_f(M, 0, b, x);
  for (int32_t i = 0; i < n; ++i)
    for (int q = 0; q < 6; ++q) z[6 * (size_t)i + q] = x[8 * (size_t)i + q];
}

/* ----------------------------------------------------------------------------------------------
 * The stress problem (stress.cpp)
 * -------------------------------------------------------------------------------------------- */

struct svxo_problem {
  int32_t n, nb;
  svxg_node* nodes;
  svxg_bond* bonds;
  svxg_material mats[SVXG_MAX_MATERIALS];
  svxg_stress_options opt;
  int assembled, pc_current, jacobi_only;
  int64_t assembly_work;
  int32_t pc_n, nfree;
  double id_scale;
  double* jinv;
  int32_t* dof;
  bsr K;
  amg M;
  int keep_levels;
  /* run state (stress.hpp:154-159) */
  int active;
  double *x, *r, *z, *p, *q;
  double rz, bn;
  int32_t iters;
};

void svxo_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int svxo_num_threads(void) { return omp_get_max_threads(); }

svxo_problem* svxo_create(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                          const svxg_material* mats) {
  svxo_problem* P = xcalloc(1, sizeof(svxo_problem));
  P->n = n;
  P->nb = nb;
  P->nodes = xcalloc((size_t)n, sizeof(svxg_node));
  P->bonds = xcalloc((size_t)nb, sizeof(svxg_bond));
  memcpy(P->nodes, nodes, sizeof(svxg_node) * (size_t)n);
  memcpy(P->bonds, bonds, sizeof(svxg_bond) * (size_t)nb);
  memcpy(P->mats, mats, sizeof(svxg_material) * SVXG_MAX_MATERIALS);
  P->opt = svxg_default_options();
  P->id_scale = 1.0;
  return P;
}

static void run_free(svxo_problem* P) {
  free(P->x);
  free(P->r);
  free(P->z);
  free(P->p);
  free(P->q);
  P->x = P->r = P->z = P->p = P->q = NULL;
  P->active = 0;
}

void svxo_destroy(svxo_problem* P) {
  if (!P) return;
  run_free(P);
  amg_clear(&P->M);
  bsr_free(&P->K);
  free(P->jinv);
  free(P->dof);
  free(P->nodes);
  free(P->bonds);
  free(P);
}

/* StressProblem::bond_matrices, stress.cpp:59-82 */
static void bond_matrices(const svxo_problem* P, const svxg_bond* b, double* D, double* Ba, double* Bb) {
  const svxg_material* A = &P->mats[b->ma];
  const svxg_material* B = &P->mats[b->mb];
  const double la = MAXD(b->la, 1e-4), lb = MAXD(b->lb, 1e-4);
  const double invE = la / A->E + lb / B->E;
  const double invG = la / A->G + lb / B->G;
  const double kt[3] = {b->area / invE, (5.0 / 6.0) * b->area / invG, (5.0 / 6.0) * b->area / invG};
  const double kr[3] = {0.8 * (b->s1 + b->s2) / invG, b->s2 / invE, b->s1 / invE};
  const v3 Q[3] = {v3_of(b->n), v3_of(b->t1), v3_of(b->t2)};
  memset(D, 0, sizeof(double) * 36);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double st = 0.0, sr = 0.0;
      for (int k = 0; k < 3; ++k) {
        st += v3_at(Q[k], r) * kt[k] * v3_at(Q[k], c);
        sr += v3_at(Q[k], r) * kr[k] * v3_at(Q[k], c);
      }
      D[r * 6 + c] = st;
      D[(3 + r) * 6 + 3 + c] = sr;
    }
  rigid_block(v3_sub(v3_of(b->p), v3_of(P->nodes[b->a].c)), Ba);
  if (b->b >= 0) rigid_block(v3_sub(v3_of(b->p), v3_of(P->nodes[b->b].c)), Bb);
}

/* StressProblem::build_matrix, stress.cpp:84-132 */
static int build_matrix(svxo_problem* P) {
  const int32_t n = P->n;
  free(P->dof);
  P->dof = xcalloc((size_t)n, sizeof(int32_t));
  P->nfree = 0;
  for (int32_t i = 0; i < n; ++i) P->dof[i] = P->nodes[i].fixed ? -1 : P->nfree++;
  builder B;
  builder_init(&B, P->nfree);
  for (int32_t i = 0; i < n; ++i)
    if (P->dof[i] >= 0) builder_block(&B, P->dof[i], P->dof[i]);
  double Dm[36], Ba[36], Bb[36];
  for (int32_t k = 0; k < P->nb; ++k) {
    svxg_bond* b = &P->bonds[k];
    b->in_k = 0;
    if (b->broken || P->nodes[b->a].gone || (b->b >= 0 && P->nodes[b->b].gone)) continue;
    b->in_k = 1;
    bond_matrices(P, b, Dm, Ba, Bb);
    const int32_t ia = P->dof[b->a];
    const int32_t ib = b->b >= 0 ? P->dof[b->b] : -1;
    if (ia >= 0) atbd_add(Ba, Dm, Ba, 1.0, builder_block(&B, ia, ia));
    if (ib >= 0) atbd_add(Bb, Dm, Bb, 1.0, builder_block(&B, ib, ib));
    if (ia >= 0 && ib >= 0) {
      atbd_add(Ba, Dm, Bb, -1.0, builder_block(&B, ia, ib));
      atbd_add(Bb, Dm, Ba, -1.0, builder_block(&B, ib, ia));
    }
  }
  bsr_free(&P->K);
  P->K = builder_finish(&B);
  double tr = 0.0;
  int32_t cnt = 0;
  for (int32_t i = 0; i < P->nfree; ++i) {
    const double* d = &P->K.val[36 * (size_t)P->K.rowptr[i]];
    const double t = d[0] + d[7] + d[14];
    if (t > 0) {
      tr += t / 3.0;
      ++cnt;
    }
  }
  P->id_scale = cnt ? tr / cnt : 1.0;
  for (int32_t i = 0; i < n; ++i) {
    const int32_t d = P->dof[i];
    if (d < 0) continue;
    double* D = &P->K.val[36 * (size_t)P->K.rowptr[d]];
    const int empty = D[0] == 0.0 && D[7] == 0.0 && D[14] == 0.0;
    if (P->nodes[i].gone || empty)
      for (int q = 0; q < 6; ++q) D[q * 7] = P->id_scale;
  }
  return 1;
}

void svxo_keep_levels(svxo_problem* P, int keep) { P->keep_levels = keep; }

/* StressProblem::assemble, stress.cpp:134-176 */
int svxo_assemble(svxo_problem* P, const svxg_stress_options* opt) {
  P->opt = opt ? *opt : svxg_default_options();
  P->assembled = 0;
  P->pc_current = 1;
  P->active = 0;
  if (!build_matrix(P)) return 0;
  P->assembly_work = 0;
  for (int32_t k = 0; k < P->nb; ++k)
    if (P->bonds[k].in_k) P->assembly_work += 48;
  v3* pos = xcalloc((size_t)P->nfree, sizeof(v3));
  for (int32_t i = 0; i < P->n; ++i)
    if (P->dof[i] >= 0) pos[P->dof[i]] = v3_of(P->nodes[i].c);
  P->jacobi_only = P->nfree < P->opt.amg_min_nodes;
  if (P->jacobi_only) {
    amg_clear(&P->M);
    P->pc_n = 0;
    free(P->jinv);
    P->jinv = xcalloc(36 * (size_t)P->nfree, sizeof(double));
    for (int32_t i = 0; i < P->nfree; ++i) {
      const double* D = &P->K.val[36 * (size_t)P->K.rowptr[i]];
      if (!inv6(D, &P->jinv[36 * (size_t)i]))
        for (int q = 0; q < 6; ++q) P->jinv[36 * (size_t)i + (size_t)(q * 7)] = 1.0 / P->id_scale;
    }
    P->assembly_work += 12 * (int64_t)P->nfree;
    P->assembled = 1;
    free(pos);
    return 1;
  }
  P->M.keep = P->keep_levels;
  const int ok = amg_build(&P->M, &P->K, pos, &P->opt.amg);
  free(pos);
  if (!ok) return 0;
  P->assembly_work += P->M.build_work;
  P->pc_n = P->nfree;
  free(P->jinv);
  P->jinv = NULL;
  P->assembled = 1;
  return 1;
}

/* StressProblem::precondition, stress.cpp:312-324 (no appended-node multigrid here) */
static void precondition(const svxo_problem* P, const double* r, double* z) {
  if (P->pc_n == P->nfree && !P->jacobi_only) {
    amg_apply(&P->M, r, z);
    return;
  }
  if (P->pc_n > 0) amg_apply(&P->M, r, z);
  for (int32_t i = P->pc_n; i < P->nfree; ++i)
    mv6(&P->jinv[36 * (size_t)(i - P->pc_n)], r + 6 * (size_t)i, z + 6 * (size_t)i);
}

void svxo_precondition(const svxo_problem* P, const double* r, double* z) { precondition(P, r, z); }
void svxo_apply_k(const svxo_problem* P, const double* x, double* y) { bsr_apply(&P->K, x, y); }

/* parallel_sum (parallel.cpp:206-227) of a . b with StressProblem::iterate's grain */
static double pdot(const double* a, const double* b, int64_t m) {
  if (m <= 0) return 0.0;
  const int64_t nch = (m + DOT_GRAIN - 1) / DOT_GRAIN;
  if (nch == 1) {
    double s = 0.0;
    for (int64_t k = 0; k < m; ++k) s += a[k] * b[k];
    return s;
  }
  double* part = xcalloc((size_t)nch, sizeof(double));
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nch; ++c) {
    const int64_t k1 = MIND(m, (c + 1) * DOT_GRAIN);
    double s = 0.0;
    for (int64_t k = c * DOT_GRAIN; k < k1; ++k) s += a[k] * b[k];
    part[c] = s;
  }
  double s = 0.0;
  for (int64_t c = 0; c < nch; ++c) s += part[c];
  free(part);
  return s;
}

/* StressProblem::begin, stress.cpp:362-401 */
void svxo_begin(svxo_problem* P, const double* f, const double* u0) {
  P->active = 0;
  if (!P->assembled && !svxo_assemble(P, &P->opt)) return;
  const size_t n = (size_t)P->n;
  const size_t m = 6 * (size_t)P->nfree;
  run_free(P);
  P->x = xcalloc(m, sizeof(double));
  P->r = xcalloc(m, sizeof(double));
  P->z = xcalloc(m, sizeof(double));
  P->p = xcalloc(m, sizeof(double));
  P->q = xcalloc(m, sizeof(double));
  double* fb = xcalloc(m, sizeof(double));
  for (size_t i = 0; i < n; ++i) {
    const int32_t d = P->dof[i];
    if (d < 0) continue;
    for (int q = 0; q < 6; ++q) {
      fb[6 * (size_t)d + q] = f[6 * i + q];
      if (u0) P->x[6 * (size_t)d + q] = u0[6 * i + q];
    }
  }
  bsr_apply(&P->K, P->x, P->q);
  double bn = 0.0;
  for (size_t k = 0; k < m; ++k) {
    P->r[k] = fb[k] - P->q[k];
    bn += fb[k] * fb[k];
  }
  free(fb);
  P->bn = sqrt(bn);
  if (!(bn > 0.0)) {
    memset(P->x, 0, sizeof(double) * m);
    memset(P->r, 0, sizeof(double) * m);
  }
  precondition(P, P->r, P->z);
  memcpy(P->p, P->z, sizeof(double) * m);
  P->rz = 0.0;
  for (size_t k = 0; k < m; ++k) P->rz += P->r[k] * P->z[k];
  P->iters = 0;
  P->active = 1;
}

/* StressProblem::iterate, stress.cpp:403-464 */
int svxo_iterate(svxo_problem* P, int32_t maxit, double rtol, svxg_pcg_result* out) {
  svxg_pcg_result res = {0, 0, 0, 0, 0.0};
  if (!P->active) {
    if (out) *out = res;
    return 0;
  }
  const int64_t m = 6 * (int64_t)P->nfree;
  double rn = sqrt(pdot(P->r, P->r, m));
  const double target = rtol * P->bn;
  if (!isfinite(P->bn) || !isfinite(rn)) {
    res.rel_res = INFINITY;
    res.breakdown = 1;
    P->active = 0;
    if (out) *out = res;
    return 0;
  }
  res.rel_res = P->bn > 0 ? rn / P->bn : 0.0;
  if (rn <= target || !(P->bn > 0) || m == 0) {
    res.converged = 1;
    if (out) *out = res;
    return 0;
  }
  for (int32_t it = 0; it < maxit; ++it) {
    bsr_apply(&P->K, P->p, P->q);
    const double pq = pdot(P->p, P->q, m);
    ++res.iters;
    ++P->iters;
    if (!(pq > 0)) {
      res.converged = 0;
      res.breakdown = 1;
      break;
    }
    const double alpha = P->rz / pq;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < m; ++k) {
      P->x[k] += alpha * P->p[k];
      P->r[k] -= alpha * P->q[k];
    }
    rn = sqrt(pdot(P->r, P->r, m));
    res.rel_res = rn / P->bn;
    if (rn <= target) {
      res.converged = 1;
      break;
    }
    precondition(P, P->r, P->z);
    const double rz1 = pdot(P->r, P->z, m);
    if (!(rz1 > 0)) {
      res.breakdown = 1;
      break;
    }
    const double beta = rz1 / P->rz;
    P->rz = rz1;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < m; ++k) P->p[k] = P->z[k] + beta * P->p[k];
  }
  if (out) *out = res;
  return 0;
}

/* StressProblem::current, stress.cpp:466-475 */
void svxo_current(const svxo_problem* P, double* u) {
  memset(u, 0, sizeof(double) * 6 * (size_t)P->n);
  if (!P->x || !P->dof) return;
  for (int32_t i = 0; i < P->n; ++i) {
    const int32_t d = P->dof[i];
    if (d < 0) continue;
    for (int q = 0; q < 6; ++q) u[6 * (size_t)i + q] = P->x[6 * (size_t)d + q];
  }
}

/* StressProblem::solve, stress.cpp:348-360 */
int svxo_solve(svxo_problem* P, const double* f, double* u, double rtol, int32_t maxit, int32_t warm,
               svxg_pcg_result* res) {
  if (!P->assembled && !svxo_assemble(P, &P->opt)) {
    if (res) {
      memset(res, 0, sizeof(*res));
      res->rel_res = INFINITY;
      res->breakdown = 1;
    }
    return 0;
  }
  svxo_begin(P, f, warm ? u : NULL);
  svxo_iterate(P, maxit < 0 ? 100000 : maxit, rtol, res);
  svxo_current(P, u);
  P->active = 0;
  return 1;
}

static double* kblock(svxo_problem* P, int32_t r, int32_t c) {
  for (int32_t k = P->K.rowptr[r]; k < P->K.rowptr[r + 1]; ++k)
    if (P->K.col[k] == c) return &P->K.val[36 * (size_t)k];
  return NULL;
}

/* StressProblem::remove_bond, stress.cpp:260-284 */
void svxo_remove_bond(svxo_problem* P, int32_t bi) {
  svxg_bond* b = &P->bonds[bi];
  b->broken = 1;
  if (!P->assembled || !b->in_k) return;
  b->in_k = 0;
  double Dm[36], Ba[36], Bb[36];
  bond_matrices(P, b, Dm, Ba, Bb);
  const int32_t ia = P->dof[b->a];
  const int32_t ib = b->b >= 0 ? P->dof[b->b] : -1;
  if (ia >= 0) atbd_add(Ba, Dm, Ba, -1.0, kblock(P, ia, ia));
  if (ib >= 0) atbd_add(Bb, Dm, Bb, -1.0, kblock(P, ib, ib));
  if (ia >= 0 && ib >= 0) {
    double* k1 = kblock(P, ia, ib);
    if (k1) atbd_add(Ba, Dm, Bb, 1.0, k1);
    double* k2 = kblock(P, ib, ia);
    if (k2) atbd_add(Bb, Dm, Ba, 1.0, k2);
  }
  if (!P->jacobi_only) P->pc_current = 0;
  if (P->jacobi_only) {
    const int32_t ds[2] = {ia, ib};
    for (int t = 0; t < 2; ++t) {
      const int32_t d = ds[t];
      if (d < 0) continue;
      const double* D = &P->K.val[36 * (size_t)P->K.rowptr[d]];
      if (!inv6(D, &P->jinv[36 * (size_t)d]))
        for (int q = 0; q < 36; ++q) P->jinv[36 * (size_t)d + q] = (q % 7 == 0) ? 1.0 / P->id_scale : 0.0;
    }
  }
  P->active = 0;
}

/* StressProblem::retire_nodes, stress.cpp:286-310 */
void svxo_retire_nodes(svxo_problem* P, const int32_t* list, int32_t count) {
  if (count <= 0) return;
  uint8_t* now = xcalloc((size_t)P->n, 1);
  for (int32_t t = 0; t < count; ++t) {
    const int32_t i = list[t];
    now[i] = P->nodes[i].gone ? 0 : 1;
    P->nodes[i].gone = 1;
  }
  for (int32_t b = 0; b < P->nb; ++b) {
    const svxg_bond* B = &P->bonds[b];
    if (now[B->a] || (B->b >= 0 && now[B->b])) svxo_remove_bond(P, b);
  }
  if (P->assembled)
    for (int32_t t = 0; t < count; ++t) {
      const int32_t i = list[t];
      const int32_t d = P->dof[i];
      if (d < 0) continue;
      if (now[i] && !P->jacobi_only) P->pc_current = 0;
      double* D = kblock(P, d, d);
      for (int q = 0; q < 36; ++q) D[q] = (q % 7 == 0) ? P->id_scale : 0.0;
      if (P->jacobi_only)
        for (int q = 0; q < 36; ++q) P->jinv[36 * (size_t)d + q] = (q % 7 == 0) ? 1.0 / P->id_scale : 0.0;
    }
  free(now);
  P->active = 0;
}

/* bond_strength, stress.cpp:14-21 */
static void bond_strength(const svxg_bond* b, double fragility, const svxg_material* mats, double S[5]) {
  const double s = b->strength / MAXD(1e-6, fragility);
  if (b->sectioned) {
    S[0] = s * b->ft;
    S[1] = s * b->fb;
    S[2] = s * b->fc;
    S[3] = s * b->coh;
    S[4] = (double)b->mu;
    return;
  }
  const svxg_material* A = &mats[b->ma];
  const svxg_material* B = &mats[b->mb];
  S[0] = s * MIND(A->ft, B->ft);
  S[1] = s * MIND(A->fb, B->fb);
  S[2] = s * MIND(A->fc, B->fc);
  S[3] = s * MIND(A->cohesion, B->cohesion);
  S[4] = MIND(A->friction, B->friction);
}

/* bond_utilization, stress.cpp:23-57 */
static double utilization(const svxg_bond* b, const svxg_bond_load* L, double fragility, const svxg_material* mats,
                          uint8_t* mode) {
  double S[5];
  bond_strength(b, fragility, mats, S);
  const double kWeakest = 1e-9;
  S[0] = MAXD(S[0], kWeakest);
  S[1] = MAXD(S[1], kWeakest);
  S[2] = MAXD(S[2], kWeakest);
  const double A = MAXD(b->area, 1e-12);
  const double sN = L->N / A;
  const double sb = (b->s2 > 0 ? fabs(L->M1) * b->c2 / b->s2 : 0.0) + (b->s1 > 0 ? fabs(L->M2) * b->c1 / b->s1 : 0.0);
  double phi_t;
  if (sN >= 0.0) {
    phi_t = sN / S[0] + sb / S[1];
  } else {
    phi_t = MAXD(0.0, sb + sN) / S[1];
  }
  const double phi_c = MAXD(0.0, sb - sN) / S[2];
  const double J = MAXD(b->s1 + b->s2, 1e-18);
  const double tau = 1.5 * sqrt(L->V1 * L->V1 + L->V2 * L->V2) / A + fabs(L->T) * b->rmax / J;
  const double cap = MAXD(S[3] + S[4] * MAXD(0.0, -sN), kWeakest);
  const double phi_s = tau / cap;
  double phi = phi_t;
  uint8_t m = SVXG_FAIL_TENSION;
  if (phi_c > phi) {
    phi = phi_c;
    m = SVXG_FAIL_CRUSH;
  }
  if (phi_s > phi) {
    phi = phi_s;
    m = SVXG_FAIL_SHEAR;
  }
  if (mode) *mode = phi > 0 ? m : SVXG_FAIL_NONE;
  return phi;
}

double svxo_utilization(const svxg_bond* b, const svxg_bond_load* L, double fragility, const svxg_material* mats,
                        uint8_t* mode) {
  return utilization(b, L, fragility, mats, mode);
}

/* ----------------------------------------------------------------------------------------------
 * Section geometry: SecAcc::finish_lattice (core/src/world/world_internal.hpp:133-232) and
 * section_strengths (world_internal.hpp:370-399), bond by bond, as World::Impl builds its bonds
 * (core/src/world/world.cpp:839-850).
 * -------------------------------------------------------------------------------------------- */

static v3 v3_scale(v3 a, double s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static v3 v3_normalized(v3 a) { /* vec.hpp:47-50 */
  const double n = sqrt(v3_dot(a, a));
  if (n > 0) return v3_scale(a, 1.0 / n);
  v3 z = {0, 0, 0};
  return z;
}
static void v3_addc(v3* a, int i, double v) {
  if (i == 0) a->x += v;
  else if (i == 1) a->y += v;
  else a->z += v;
}
static void frame_of(v3 n, v3* t1, v3* t2) { /* world_internal.hpp:64-69 */
  const double ax = fabs(n.x), ay = fabs(n.y), az = fabs(n.z);
  v3 e = {0, 0, 1};
  if (ax <= ay && ax <= az) { e.x = 1; e.z = 0; }
  else if (ay <= az) { e.y = 1; e.z = 0; }
  *t1 = v3_normalized(v3_cross(n, e));
  *t2 = v3_cross(n, *t1);
}
static v3 face_centre(const svxg_face* F, double h) {
  v3 x = {h * F->x, h * F->y, h * F->z};
  v3_addc(&x, F->axis, 0.5 * h);
  return x;
}
static const svxg_material* vox_material(const svxg_material* mats, uint8_t a, uint8_t b) {
  /* grid.hpp:33-36: a side that is air takes the other's material */
  const int id = (a != 0 ? (a & 0x7F) : (b & 0x7F)) - 1;
  return &mats[id >= 0 && id < SVXG_MAX_MATERIALS ? id : 0];
}

/* LatticeXf::to / dir_to (rigid.hpp:91-93) with M3 * V3 (vec.hpp:63-66) */
static v3 xf_dir(const svxg_lattice* X, v3 d) {
  if (!X || X->identity) return d;
  const double* R = X->R;
  v3 r = {R[0] * d.x + R[1] * d.y + R[2] * d.z, R[3] * d.x + R[4] * d.y + R[5] * d.z,
          R[6] * d.x + R[7] * d.y + R[8] * d.z};
  return r;
}
static v3 xf_to(const svxg_lattice* X, v3 s) {
  if (!X || X->identity) return s;
  const v3 r = xf_dir(X, s);
  v3 o = {X->off[0] + r.x, X->off[1] + r.y, X->off[2] + r.z};
  return o;
}
/* junction_point (world_internal.hpp:94-103) with push 0 */
static v3 junction_point(const int32_t* v, int face, int sub, int32_t S, double h) {
  const int a = face >> 1, a1 = (a + 1) % 3, a2 = (a + 2) % 3;
  const double sg = (face & 1) ? 1.0 : -1.0;
  const int i = sub / S, j = sub % S;
  v3 s = {h * v[0], h * v[1], h * v[2]};
  v3_addc(&s, a, sg * (0.5 * h + 0.0));
  v3_addc(&s, a1, ((i + 0.5) / (double)S - 0.5) * h);
  v3_addc(&s, a2, ((j + 0.5) / (double)S - 0.5) * h);
  return s;
}

/* SecAcc::finish_general (world_internal.hpp:237-352) and section_strengths_general
 * (world_internal.hpp:404-441): faces of a placed lattice and junction samples, each a small
 * square at a point with a normal, projected onto the plane normal to their mean normal. */
static svxg_bond finish_general(const svxg_node* nodes, const svxg_section* S, const svxg_face* F,
                                const svxg_junction* J, const svxg_lattice* lats, int32_t Sj,
                                const svxg_material* mats) {
  svxg_bond B;
  memset(&B, 0, sizeof(B));
  B.a = S->a;
  B.b = S->b;
  B.ma = S->ma;
  B.mb = S->mb;
  const int32_t nf = S->faces, nj = S->junctions, ne = nf + nj;
  B.faces = ne;
  v3* xs = (v3*)malloc(sizeof(v3) * (size_t)(ne > 0 ? ne : 1));
  v3* nk = (v3*)malloc(sizeof(v3) * (size_t)(ne > 0 ? ne : 1));
  double* ar = (double*)malloc(sizeof(double) * (size_t)(ne > 0 ? ne : 1));
  double* sd = (double*)malloc(sizeof(double) * (size_t)(ne > 0 ? ne : 1));
  double* ws = (double*)malloc(sizeof(double) * (size_t)(ne > 0 ? ne : 1));
  const double h = S->h, A1 = h * h;
  const svxg_lattice* X = lats ? &lats[S->grid] : NULL;
  for (int32_t k = 0; k < nf; ++k) {
    v3 x = {h * F[k].x, h * F[k].y, h * F[k].z};
    v3_addc(&x, F[k].axis, 0.5 * h);
    xs[k] = xf_to(X, x);
    v3 n0 = {0, 0, 0};
    v3_addc(&n0, F[k].axis, (double)F[k].sign);
    nk[k] = xf_dir(X, n0);
    ar[k] = A1;
    sd[k] = h;
  }
  for (int32_t q = 0; q < nj; ++q) {
    const svxg_junction* s = &J[q];
    const svxg_lattice* Xs = &lats[s->vg];
    const double hs = Xs->h, sj = hs / (double)(Sj > 1 ? Sj : 1);
    const int32_t k = nf + q;
    xs[k] = xf_to(Xs, junction_point(s->v, s->face, s->sub, Sj, hs));
    v3 fn = {0, 0, 0};
    v3_addc(&fn, s->face >> 1, (s->face & 1) ? 1.0 : -1.0);
    nk[k] = v3_scale(xf_dir(Xs, fn), (double)s->sign);
    ar[k] = sj * sj * (double)s->weight;
    sd[k] = sj;
  }
  double atot = 0.0;
  for (int32_t k = 0; k < ne; ++k) atot += ar[k];
  const v3 ca = v3_of(nodes[S->a].c);
  const int has_b = S->b >= 0;
  const v3 cb = has_b ? v3_of(nodes[S->b].c) : ca;
  v3 n = {0, 0, 0};
  if (has_b || nj) {
    for (int32_t k = 0; k < ne; ++k) {
      const v3 t = v3_scale(nk[k], ar[k]);
      n.x += t.x;
      n.y += t.y;
      n.z += t.z;
    }
    const double tiny = 1e-12 * atot * atot;
    if (v3_dot(n, n) <= tiny && has_b) n = v3_sub(cb, ca);
    if (v3_dot(n, n) <= tiny) { n.x = 0; n.y = 0; n.z = 1; }
    n = v3_normalized(n);
  } else {
    v3 e = {0, 0, 0};
    v3_addc(&e, S->axis, (double)S->sign);
    n = xf_dir(X, e);
  }
  v3 t1, t2;
  frame_of(n, &t1, &t2);
  double W = 0.0;
  v3 pc = {0, 0, 0};
  for (int32_t k = 0; k < ne; ++k) {
    ws[k] = ar[k] * MAXD(0.05, fabs(v3_dot(n, nk[k])));
    W += ws[k];
    pc.x += xs[k].x * ws[k];
    pc.y += xs[k].y * ws[k];
    pc.z += xs[k].z * ws[k];
  }
  pc = v3_scale(pc, 1.0 / W);
  {
    double s11 = 0.0, s22 = 0.0, s12 = 0.0;
    for (int32_t k = 0; k < ne; ++k) {
      const v3 d = v3_sub(xs[k], pc);
      const double y1 = v3_dot(d, t1), y2 = v3_dot(d, t2);
      s11 += ws[k] * y1 * y1;
      s22 += ws[k] * y2 * y2;
      s12 += ws[k] * y1 * y2;
    }
    if (fabs(s12) > 1e-9 * (s11 + s22)) {
      const double half = 0.5 * (s11 - s22);
      const double l1 = 0.5 * (s11 + s22) + sqrt(half * half + s12 * s12);
      double e1 = s12, e2 = l1 - s11;
      if (fabs(l1 - s22) > fabs(e2)) {
        e1 = l1 - s22;
        e2 = s12;
      }
      const double en = sqrt(e1 * e1 + e2 * e2);
      if (en > 0.0) {
        e1 /= en;
        e2 /= en;
        const v3 u1 = {t1.x * e1 + t2.x * e2, t1.y * e1 + t2.y * e2, t1.z * e1 + t2.z * e2};
        const v3 u2 = {t2.x * e1 - t1.x * e2, t2.y * e1 - t1.y * e2, t2.z * e1 - t1.z * e2};
        t1 = u1;
        t2 = u2;
      }
    }
  }
  B.n.x = n.x; B.n.y = n.y; B.n.z = n.z;
  B.t1.x = t1.x; B.t1.y = t1.y; B.t1.z = t1.z;
  B.t2.x = t2.x; B.t2.y = t2.y; B.t2.z = t2.z;
  B.p.x = pc.x; B.p.y = pc.y; B.p.z = pc.z;
  B.area = MAXD(W, 0.25 * atot);
  double s1 = 0.0, s2 = 0.0, m1 = 0.0, m2 = 0.0, own = 0.0;
  for (int32_t k = 0; k < ne; ++k) {
    const v3 d = v3_sub(xs[k], pc);
    const double y1 = v3_dot(d, t1), y2 = v3_dot(d, t2);
    s1 += ws[k] * y1 * y1;
    s2 += ws[k] * y2 * y2;
    m1 = MAXD(m1, fabs(y1) + 0.5 * sd[k]);
    m2 = MAXD(m2, fabs(y2) + 0.5 * sd[k]);
    own += ws[k] * sd[k] * sd[k];
  }
  own /= W;
  B.s1 = s1 + B.area * own / 12.0;
  B.s2 = s2 + B.area * own / 12.0;
  B.c1 = m1;
  B.c2 = m2;
  B.rmax = sqrt(B.c1 * B.c1 + B.c2 * B.c2);
  if (has_b) {
    const v3 d = v3_sub(cb, ca);
    const double L = MAXD(MAXD(fabs(v3_dot(d, n)), 0.5 * sqrt(v3_dot(d, d))), 0.5 * h);
    const double x = v3_dot(v3_sub(pc, ca), n), lo = 0.1 * L, hi = 0.9 * L;
    B.la = x < lo ? lo : (hi < x ? hi : x);
    B.lb = L - B.la;
  } else {
    B.la = MAXD(0.25 * h, v3_dot(v3_sub(pc, ca), n));
    B.lb = 0.5 * h;
  }
  B.strength = MIND(S->strength_a, S->strength_b);
  if (S->sectioned) {
    double ft = 0, fb = 0, fc = 0, coh = 0, mu = 0, wsum = 0;
    const double sw = 1.0 / (double)(Sj * Sj > 1 ? Sj * Sj : 1);
    for (int32_t k = 0; k < ne; ++k) {
      uint8_t va, vb, da, db;
      double w;
      if (k < nf) {
        va = F[k].vox_lo; vb = F[k].vox_hi; da = F[k].damage_lo; db = F[k].damage_hi;
        w = 1.0;
      } else {
        const svxg_junction* s = &J[k - nf];
        va = s->vox_v; da = s->damage_v;
        if (s->kind == 1) { vb = va; db = da; } else { vb = s->vox_o; db = s->damage_o; }
        w = sw * (double)1.0f;
      }
      const svxg_material* A = vox_material(mats, va, vb);
      const svxg_material* M = vox_material(mats, vb, va);
      const int dm = da > db ? da : db;
      const double cond = MAXD(1e-6, 1.0 - (double)dm / 255.0);
      ft += w * cond * MIND(A->ft, M->ft);
      fb += w * cond * MIND(A->fb, M->fb);
      fc += w * cond * MIND(A->fc, M->fc);
      coh += w * cond * MIND(A->cohesion, M->cohesion);
      mu += w * MIND(A->friction, M->friction);
      wsum += w;
    }
    if (ne > 0 && wsum > 0.0) {
      const double w = 1.0 / wsum;
      B.sectioned = 1;
      B.ft = (float)(ft * w);
      B.fb = (float)(fb * w);
      B.fc = (float)(fc * w);
      B.coh = (float)(coh * w);
      B.mu = (float)(mu * w);
    }
  }
  free(xs);
  free(nk);
  free(ar);
  free(sd);
  free(ws);
  return B;
}

void svxo_build_bonds(const svxg_node* nodes, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                      const svxg_junction* juncs, const svxg_lattice* lats, int32_t samples,
                      const svxg_material* mats, svxg_bond* out) {
  for (int32_t k = 0; k < nb; ++k) {
    const svxg_section* S = &secs[k];
    if (S->junctions > 0 || (lats && !lats[S->grid].identity)) {  /* SecAcc::finish (world_internal.hpp:130-133) */
      out[k] = finish_general(nodes, S, faces + S->first_face, juncs ? juncs + S->first_junction : NULL, lats,
                              samples, mats);
      out[k].tag = k;
      continue;
    }
    const svxg_face* F = faces + S->first_face;
    const int32_t nf = S->faces;
    svxg_bond B;
    memset(&B, 0, sizeof(B));
    B.a = S->a;
    B.b = S->b;
    B.ma = S->ma;
    B.mb = S->mb;
    B.faces = nf;
    const double h = S->h, A1 = h * h;
    const v3 ca = v3_of(nodes[S->a].c);
    const int has_b = S->b >= 0;
    const v3 cb = has_b ? v3_of(nodes[S->b].c) : ca;
    v3 n = {0, 0, 0};
    if (has_b) {
      for (int32_t f = 0; f < nf; ++f) v3_addc(&n, F[f].axis, (double)F[f].sign);
      if (v3_dot(n, n) < 1e-12) n = v3_sub(cb, ca);
      if (v3_dot(n, n) < 1e-12) { n.x = 0; n.y = 0; n.z = 1; }
      n = v3_normalized(n);
    } else {
      v3_addc(&n, S->axis, (double)S->sign);
    }
    v3 t1, t2;
    frame_of(n, &t1, &t2);
    double W = 0.0;
    v3 pc = {0, 0, 0};
    for (int32_t f = 0; f < nf; ++f) {
      const v3 x = face_centre(&F[f], h);
      const double w = A1 * MAXD(0.05, fabs(v3_at(n, F[f].axis)));
      W += w;
      pc.x += x.x * w;
      pc.y += x.y * w;
      pc.z += x.z * w;
    }
    pc = v3_scale(pc, 1.0 / W);
    {
      double s11 = 0.0, s22 = 0.0, s12 = 0.0;
      for (int32_t f = 0; f < nf; ++f) {
        const v3 d = v3_sub(face_centre(&F[f], h), pc);
        const double w = A1 * MAXD(0.05, fabs(v3_at(n, F[f].axis)));
        const double y1 = v3_dot(d, t1), y2 = v3_dot(d, t2);
        s11 += w * y1 * y1;
        s22 += w * y2 * y2;
        s12 += w * y1 * y2;
      }
      if (fabs(s12) > 1e-9 * (s11 + s22)) {
        const double half = 0.5 * (s11 - s22);
        const double l1 = 0.5 * (s11 + s22) + sqrt(half * half + s12 * s12);
        double e1 = s12, e2 = l1 - s11;
        if (fabs(l1 - s22) > fabs(e2)) {
          e1 = l1 - s22;
          e2 = s12;
        }
        const double en = sqrt(e1 * e1 + e2 * e2);
        if (en > 0.0) {
          e1 /= en;
          e2 /= en;
          const v3 u1 = {t1.x * e1 + t2.x * e2, t1.y * e1 + t2.y * e2, t1.z * e1 + t2.z * e2};
          const v3 u2 = {t2.x * e1 - t1.x * e2, t2.y * e1 - t1.y * e2, t2.z * e1 - t1.z * e2};
          t1 = u1;
          t2 = u2;
        }
      }
    }
    B.n.x = n.x; B.n.y = n.y; B.n.z = n.z;
    B.t1.x = t1.x; B.t1.y = t1.y; B.t1.z = t1.z;
    B.t2.x = t2.x; B.t2.y = t2.y; B.t2.z = t2.z;
    B.p.x = pc.x; B.p.y = pc.y; B.p.z = pc.z;
    B.area = MAXD(W, 0.25 * nf * A1);
    double s1 = 0.0, s2 = 0.0, m1 = 0.0, m2 = 0.0;
    for (int32_t f = 0; f < nf; ++f) {
      const v3 d = v3_sub(face_centre(&F[f], h), pc);
      const double w = A1 * MAXD(0.05, fabs(v3_at(n, F[f].axis)));
      const double y1 = v3_dot(d, t1), y2 = v3_dot(d, t2);
      s1 += w * y1 * y1;
      s2 += w * y2 * y2;
      m1 = MAXD(m1, fabs(y1));
      m2 = MAXD(m2, fabs(y2));
    }
    B.s1 = s1 + B.area * A1 / 12.0;
    B.s2 = s2 + B.area * A1 / 12.0;
    B.c1 = m1 + 0.5 * h;
    B.c2 = m2 + 0.5 * h;
    B.rmax = sqrt(B.c1 * B.c1 + B.c2 * B.c2);
    if (has_b) {
      const v3 d = v3_sub(cb, ca);
      const double L = MAXD(MAXD(fabs(v3_dot(d, n)), 0.5 * sqrt(v3_dot(d, d))), 0.5 * h);
      const double x = v3_dot(v3_sub(pc, ca), n), lo = 0.1 * L, hi = 0.9 * L;
      B.la = x < lo ? lo : (hi < x ? hi : x);
      B.lb = L - B.la;
    } else {
      B.la = MAXD(0.25 * h, v3_dot(v3_sub(pc, ca), n));
      B.lb = 0.5 * h;
    }
    B.strength = MIND(S->strength_a, S->strength_b);
    if (S->sectioned && nf > 0) {
      double ft = 0, fb = 0, fc = 0, coh = 0, mu = 0;
      for (int32_t f = 0; f < nf; ++f) {
        const svxg_material* A = vox_material(mats, F[f].vox_lo, F[f].vox_hi);
        const svxg_material* M = vox_material(mats, F[f].vox_hi, F[f].vox_lo);
        const int dm = F[f].damage_lo > F[f].damage_hi ? F[f].damage_lo : F[f].damage_hi;
        const double cond = MAXD(1e-6, 1.0 - (double)dm / 255.0);
        ft += cond * MIND(A->ft, M->ft);
        fb += cond * MIND(A->fb, M->fb);
        fc += cond * MIND(A->fc, M->fc);
        coh += cond * MIND(A->cohesion, M->cohesion);
        mu += MIND(A->friction, M->friction);
      }
      const double w = 1.0 / (double)nf;
      B.sectioned = 1;
      B.ft = (float)(ft * w);
      B.fb = (float)(fb * w);
      B.fc = (float)(fc * w);
      B.coh = (float)(coh * w);
      B.mu = (float)(mu * w);
    }
    B.tag = k;
    out[k] = B;
  }
}

/* StressProblem::bond_load, stress.cpp:477-502 */
static svxg_bond_load bond_load(const svxo_problem* P, int32_t bi, const double* u) {
  const svxg_bond* b = &P->bonds[bi];
  const svxg_material* A = &P->mats[b->ma];
  const svxg_material* B = &P->mats[b->mb];
  double Ba[36], Bb[36];
  rigid_block(v3_sub(v3_of(b->p), v3_of(P->nodes[b->a].c)), Ba);
  double xa[6] = {0, 0, 0, 0, 0, 0}, xb[6] = {0, 0, 0, 0, 0, 0};
  if (!P->nodes[b->a].fixed) mv6(Ba, &u[6 * (size_t)b->a], xa);
  if (b->b >= 0) {
    rigid_block(v3_sub(v3_of(b->p), v3_of(P->nodes[b->b].c)), Bb);
    if (!P->nodes[b->b].fixed) mv6(Bb, &u[6 * (size_t)b->b], xb);
  }
  const v3 dt = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
  const v3 dr = {xb[3] - xa[3], xb[4] - xa[4], xb[5] - xa[5]};
  const double la = MAXD(b->la, 1e-4), lb = MAXD(b->lb, 1e-4);
  const double invE = la / A->E + lb / B->E;
  const double invG = la / A->G + lb / B->G;
  svxg_bond_load L;
  L.N = b->area / invE * v3_dot(dt, v3_of(b->n));
  L.V1 = (5.0 / 6.0) * b->area / invG * v3_dot(dt, v3_of(b->t1));
  L.V2 = (5.0 / 6.0) * b->area / invG * v3_dot(dt, v3_of(b->t2));
  L.T = 0.8 * (b->s1 + b->s2) / invG * v3_dot(dr, v3_of(b->n));
  L.M1 = b->s2 / invE * v3_dot(dr, v3_of(b->t1));
  L.M2 = b->s1 / invE * v3_dot(dr, v3_of(b->t2));
  return L;
}

void svxo_judge(const svxo_problem* P, const double* u, double fragility, svxg_bond_load* loads, double* phi,
                uint8_t* mode) {
  for (int32_t k = 0; k < P->nb; ++k) {
    const svxg_bond_load L = bond_load(P, k, u);
    uint8_t md = 0;
    const double ph = utilization(&P->bonds[k], &L, fragility, P->mats, &md);
    if (loads) loads[k] = L;
    if (phi) phi[k] = ph;
    if (mode) mode[k] = md;
  }
}

/* bond_utilization of every bond of the problem under the given loads (one per bond) */
void svxo_utilization_many(const svxo_problem* P, const svxg_bond_load* loads, double fragility, double* phi,
                           uint8_t* mode) {
  for (int32_t k = 0; k < P->nb; ++k) {
    uint8_t md = 0;
    phi[k] = utilization(&P->bonds[k], &loads[k], fragility, P->mats, &md);
    if (mode) mode[k] = md;
  }
}

/* A caller writing bonds[b].broken (the public member), as the piece rounds do for a chip's inner
 * bonds after retiring it (core/src/world/world_pieces.cpp:800-802). */
void svxo_set_broken(svxo_problem* P, int32_t b, int v) { P->bonds[b].broken = (uint8_t)(v != 0); }

/* StressProblem::invalidate / assembled / preconditioner_current (stress.hpp:83-91) */
void svxo_invalidate(svxo_problem* P) {
  P->assembled = 0;
  P->active = 0;
}
int svxo_assembled(const svxo_problem* P) { return P->assembled; }
int svxo_preconditioner_current(const svxo_problem* P) { return P->assembled && P->pc_current; }

void svxo_get_info(const svxo_problem* P, svxo_info* info) {
  memset(info, 0, sizeof(*info));
  info->nfree = P->nfree;
  info->block_jacobi = P->jacobi_only;
  info->levels = P->M.nlev;
  info->chol_n = P->M.chol_n;
  for (int32_t l = 0; l < P->M.nlev; ++l) {
    info->level_sizes[l] = P->M.lv[l].A.n;
    info->level_blocks[l] = P->M.lv[l].A.nnzb;
    info->level_blocks[P->M.nlev + l] = P->M.lv[l].pnnz;
  }
  info->matrix_blocks = P->K.nnzb;
  info->work_per_iteration = 2 * P->K.nnzb + P->M.work;
  info->assembly_work = P->assembly_work;
  info->work_per_apply = P->M.work;
  info->build_work = P->M.build_work;
}

void svxo_bond_flags(const svxo_problem* P, uint8_t* broken, uint8_t* in_k) {
  for (int32_t k = 0; k < P->nb; ++k) {
    if (broken) broken[k] = P->bonds[k].broken;
    if (in_k) in_k[k] = P->bonds[k].in_k;
  }
}

void svxo_matrix_dims(const svxo_problem* P, int32_t* nfree, int64_t* nnzb) {
  *nfree = P->K.n;
  *nnzb = P->K.nnzb;
}

void svxo_matrix(const svxo_problem* P, int32_t* dof, int32_t* rowptr, int32_t* col, double* val, double* id_scale) {
  if (dof) memcpy(dof, P->dof, sizeof(int32_t) * (size_t)P->n);
  if (rowptr) memcpy(rowptr, P->K.rowptr, sizeof(int32_t) * ((size_t)P->K.n + 1));
  if (col) memcpy(col, P->K.col, sizeof(int32_t) * (size_t)P->K.nnzb);
  if (val) memcpy(val, P->K.val, sizeof(double) * 36 * (size_t)P->K.nnzb);
  if (id_scale) *id_scale = P->id_scale;
}

int32_t svxo_levels(const svxo_problem* P) { return P->M.nlev; }

void svxo_level_dims(const svxo_problem* P, int32_t l, int32_t* n, int64_t* nnzb, int64_t* pnnz) {
  const level* L = &P->M.lv[l];
  *n = L->A.n;
  *nnzb = L->A.nnzb;
  *pnnz = L->pnnz;
}

void svxo_level_get(const svxo_problem* P, int32_t l, int32_t* rowptr, int32_t* col, double* val, double* dinv,
                    int32_t* parent, int32_t* prow, int32_t* pcol, double* pval, double* pos, double* lmax) {
  const level* L = &P->M.lv[l];
  const size_t n = (size_t)L->A.n;
  if (rowptr) memcpy(rowptr, L->A.rowptr, sizeof(int32_t) * (n + 1));
  if (col) memcpy(col, L->A.col, sizeof(int32_t) * (size_t)L->A.nnzb);
  if (val && L->A.val) memcpy(val, L->A.val, sizeof(double) * 36 * (size_t)L->A.nnzb);
  if (dinv && L->Dinv) memcpy(dinv, L->Dinv, sizeof(double) * 36 * n);
  if (parent && L->parent) memcpy(parent, L->parent, sizeof(int32_t) * n);
  if (prow && L->Prow) memcpy(prow, L->Prow, sizeof(int32_t) * (n + 1));
  if (pcol && L->Pcol) memcpy(pcol, L->Pcol, sizeof(int32_t) * (size_t)L->pnnz);
  if (pval && L->Pval) memcpy(pval, L->Pval, sizeof(double) * 36 * (size_t)L->pnnz);
  if (pos && L->pos)
    for (size_t i = 0; i < n; ++i) {
      pos[3 * i] = L->pos[i].x;
      pos[3 * i + 1] = L->pos[i].y;
      pos[3 * i + 2] = L->pos[i].z;
    }
  if (lmax) {
    amg tmp = P->M;
    *lmax = estimate_lmax(&tmp, L);
  }
}

int32_t svxo_chol_n(const svxo_problem* P) { return P->M.chol_n; }
void svxo_chol(const svxo_problem* P, double* out) {
  memcpy(out, P->M.chol, sizeof(double) * (size_t)P->M.chol_n * (size_t)P->M.chol_n);
}

double svxo_seq_sum(const double* a, int64_t n) {
  double s = 0.0;
  for (int64_t k = 0; k < n; ++k) s += a[k];
  return s;
}

/* ---- loads (the checker of the library's load builders) --------------------------------------- */

static v3 v3_add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
/* M3 * V3 and M3 * M3, row-major (core/include/svx/base/vec.hpp:63-72) */
static v3 m3_v(const double* A, v3 v) {
  v3 r = {A[0] * v.x + A[1] * v.y + A[2] * v.z, A[3] * v.x + A[4] * v.y + A[5] * v.z,
          A[6] * v.x + A[7] * v.y + A[8] * v.z};
  return r;
}
static void m3_m(const double* A, const double* B, double* R) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
}
/* R * A * R^T, left to right as the reference writes it: (R * A) * Rt */
static void m3_conj(const double* R, const double* A, const double* Rt, double* out) {
  double T[9];
  m3_m(R, A, T);
  m3_m(T, Rt, out);
}

void svxo_structure_loads(int32_t n, const double* weight, const double* ext, double* f) {
  /* World::Impl::load_vector, core/src/world/world.cpp:966-974 */
  for (int64_t i = 0; i < n; ++i) {
    for (int q = 0; q < 6; ++q) f[6 * i + q] = 0.0;
    f[6 * i + 2] = -weight[i];
    for (int q = 0; q < 6; ++q) f[6 * i + q] += ext ? ext[6 * i + q] : 0.0;
  }
}

int32_t svxo_pin_reference(svxg_node* nodes, int32_t n, svxg_v3 com) {
  /* pin_reference, core/src/world/world_pieces.cpp:313-326 */
  int32_t pin = 0;
  double best = 1e300;
  for (int32_t i = 0; i < n; ++i) {
    nodes[i].fixed = 0;
    v3 d = v3_sub(v3_of(nodes[i].c), v3_of(com));
    double d2 = v3_dot(d, d);
    if (d2 < best) {
      best = d2;
      pin = i;
    }
  }
  if (n > 0) nodes[pin].fixed = 1;
  return n > 0 ? pin : -1;
}

void svxo_body_loads(const svxg_body_state* b, const svxg_node* nodes, int32_t n, const svxg_v3* node_com,
                     const double* node_mass, const double* node_inertia, const svxg_point_force* forces,
                     int32_t nforces, int32_t inertia, double* f) {
  /* World::Impl::body_stress_run's loads, core/src/world/world_pieces.cpp:566-603 */
  const double* q = b->q;
  /* to_matrix (vec.hpp:111-120) */
  const double xx = q[0] * q[0], yy = q[1] * q[1], zz = q[2] * q[2];
  const double xy = q[0] * q[1], xz = q[0] * q[2], yz = q[1] * q[2];
  const double wx = q[3] * q[0], wy = q[3] * q[1], wz = q[3] * q[2];
  const double R[9] = {1 - 2 * (yy + zz), 2 * (xy - wz), 2 * (xz + wy), 2 * (xy + wz), 1 - 2 * (xx + zz),
                       2 * (yz - wx), 2 * (xz - wy), 2 * (yz + wx), 1 - 2 * (xx + yy)};
  double Rt[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Rt[3 * r + c] = R[3 * c + r];
  for (int64_t k = 0; k < 6 * (int64_t)n; ++k) f[k] = 0.0;
  const v3 g = {0, 0, -b->gravity};
  const v3 x = v3_of(b->x), bc = v3_of(b->com), w = v3_of(b->w);
  if (inertia) {
    v3 Ft = {0, 0, 0}, tau = {0, 0, 0};
    for (int32_t k = 0; k < nforces; ++k) {
      Ft = v3_add(Ft, v3_of(forces[k].F));
      tau = v3_add(tau, v3_cross(v3_sub(v3_of(forces[k].p), x), v3_of(forces[k].F)));
    }
    double Iw[9], Iwi[9];
    m3_conj(R, b->inertia, Rt, Iw);
    m3_conj(R, b->inv_inertia, Rt, Iwi);
    const v3 a = v3_add(v3_scale(Ft, b->inv_mass), g);
    const v3 alpha = m3_v(Iwi, v3_sub(tau, v3_cross(w, m3_v(Iw, w))));
    for (int32_t i = 0; i < n; ++i) {
      const v3 rw = m3_v(R, v3_sub(v3_of(node_com[i]), bc));
      const v3 ai = v3_add(v3_add(a, v3_cross(alpha, rw)), v3_cross(w, v3_cross(w, rw)));
      const v3 Fi = m3_v(Rt, v3_scale(v3_sub(g, ai), node_mass[i]));
      double Ii[9];
      m3_conj(R, node_inertia + 9 * (int64_t)i, Rt, Ii);
      const v3 Mi = m3_v(Rt, v3_scale(v3_add(m3_v(Ii, alpha), v3_cross(w, m3_v(Ii, w))), -1.0));
      double* fi = f + 6 * (int64_t)i;
      fi[0] += Fi.x;
      fi[1] += Fi.y;
      fi[2] += Fi.z;
      fi[3] += Mi.x;
      fi[4] += Mi.y;
      fi[5] += Mi.z;
    }
  }
  for (int32_t k = 0; k < nforces; ++k) {
    const int32_t i = forces[k].node;
    if (i < 0 || i >= n) continue;
    /* Body::to_shape (phys/rigid.hpp:206) with rotate_inv = rotate by conj(q) (vec.hpp:105-110) */
    const v3 u = {-q[0], -q[1], -q[2]};
    const v3 d = v3_sub(v3_of(forces[k].p), x);
    const v3 t = v3_scale(v3_cross(u, d), 2.0);
    const v3 at = v3_add(bc, v3_add(v3_add(d, v3_scale(t, q[3])), v3_cross(u, t)));
    /* StressProblem::add_force (core/src/stress/stress.cpp:504-513) */
    const v3 F = m3_v(Rt, v3_of(forces[k].F));
    double* fi = f + 6 * (int64_t)i;
    fi[0] += F.x;
    fi[1] += F.y;
    fi[2] += F.z;
    const v3 M = v3_cross(v3_sub(at, v3_of(nodes[i].c)), F);
    fi[3] += M.x;
    fi[4] += M.y;
    fi[5] += M.z;
  }
}
