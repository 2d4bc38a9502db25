// blk6.cuh - exact 6x6 block arithmetic of the stress solve's setup (host and device).
//
// Every function here evaluates its sums in the same order as the reference's
// (core/src/solve/amg.cpp:47-170, amg.hpp:132-161, core/src/stress/stress.cpp:59-82) and is
// compiled without multiply-add contraction (device translation units named exact_*.cu are
// built with -fmad=false; host tests with -ffp-contract=off), so the device's K, aggregates,
// prolongations and coarse operators equal the reference's value for value. The same source is
// compiled on the host by the tests to check that claim without a GPU.
#pragma once

#include <math.h>
#include <stdint.h>

#include "svxg_types.h"

#if defined(__CUDACC__)
#define SVXG_HD __host__ __device__ __forceinline__
#else
#define SVXG_HD inline
#endif

namespace svxg {

// std::max / std::min as <algorithm> evaluates them (NaN order included)
SVXG_HD double maxd(double a, double b) { return a < b ? b : a; }
SVXG_HD double mind(double a, double b) { return b < a ? b : a; }

struct V3d {
  double x, y, z;
};
SVXG_HD V3d sub3(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
SVXG_HD double dot3(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SVXG_HD double at3(V3d a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
SVXG_HD V3d v3of(const svxg_v3& a) { return {a.x, a.y, a.z}; }

// blk6::rigid_block (amg.cpp:143-153): P = [[I, -[r]x], [0, I]]
SVXG_HD void rigid_block(V3d r, double* P) {
  for (int i = 0; i < 36; ++i) P[i] = 0.0;
  for (int i = 0; i < 6; ++i) P[i * 6 + i] = 1.0;
  P[0 * 6 + 4] = r.z;
  P[0 * 6 + 5] = -r.y;
  P[1 * 6 + 3] = -r.z;
  P[1 * 6 + 5] = r.x;
  P[2 * 6 + 3] = r.y;
  P[2 * 6 + 4] = -r.x;
}

// The bond's local stiffness D = Q^T diag(kt, kr) Q as its two 3x3 blocks (the rest of the 6x6 is
// zero), stress.cpp:59-79.
struct BondStiffness {
  double Dt[9], Dr[9];
};

SVXG_HD void bond_stiffness(const svxg_bond& b, const svxg_material* mats, BondStiffness& S) {
  const svxg_material& A = mats[b.ma];
  const svxg_material& B = mats[b.mb];
  const double la = maxd(b.la, 1e-4), lb = maxd(b.lb, 1e-4);
  const double invE = la / A.E + lb / B.E;
  const double invG = la / A.G + lb / B.G;
  const double kt[3] = {b.area / invE, (5.0 / 6.0) * b.area / invG, (5.0 / 6.0) * b.area / invG};
  const double kr[3] = {0.8 * (b.s1 + b.s2) / invG, b.s2 / invE, b.s1 / invE};
  const V3d Q[3] = {v3of(b.n), v3of(b.t1), v3of(b.t2)};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double st = 0.0, sr = 0.0;
      for (int k = 0; k < 3; ++k) {
        st += at3(Q[k], r) * kt[k] * at3(Q[k], c);
        sr += at3(Q[k], r) * kr[k] * at3(Q[k], c);
      }
      S.Dt[r * 3 + c] = st;
      S.Dr[r * 3 + c] = sr;
    }
}

// C += s A^T (D B) with A = rigid_block(ra), B = rigid_block(rb) and D held as its two 3x3
// diagonal blocks: blk6::atbd_add (amg.cpp:155-170) loop for loop, D's zero blocks read as 0.
SVXG_HD void atbd_add_rigid(V3d ra, const BondStiffness& S, V3d rb, double s, double* C) {
  double A[36], B[36];
  rigid_block(ra, A);
  rigid_block(rb, B);
  // T = D B: rows 0-2 = [Dt, Dt R_b], rows 3-5 = [0, Dr]; the loop's sum over k for each entry
  double T[36];
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) {
        const bool rt = r < 3, kt = k < 3;
        const double d = (rt == kt) ? (rt ? S.Dt[r * 3 + k] : S.Dr[(r - 3) * 3 + (k - 3)]) : 0.0;
        acc += d * B[k * 6 + c];
      }
      T[r * 6 + c] = acc;
    }
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) acc += A[k * 6 + r] * T[k * 6 + c];
      C[r * 6 + c] += s * acc;
    }
}

// The same as atbd_add_rigid with the products by the rigid blocks' exact zeros and ones left out.
// Every entry keeps the full loops' sequence of nonzero roundings: a zero product added to a sum
// leaves its value (x + 0 = x; only a zero's sign can differ), and x * 1 = x, so each result equals
// atbd_add's value for value (checked entry by entry against the full loops by the tests).
//   T = D B:      rows 0-2: [Dt, Dt R_b] (R_b the skew block of rb), rows 3-5: [0, Dr]
//   A^T T:        rows 0-2: T's rows 0-2; row 3 + i: the two nonzero R_a(k, i) T[k] terms in k
//                 order, then T[3 + i]
SVXG_HD void atbd_add_rigid_fast(V3d ra, const BondStiffness& S, V3d rb, double s, double* C) {
  const double* Dt = S.Dt;
  const double* Dr = S.Dr;
  double T[36];
  for (int r = 0; r < 3; ++r) {
    const double d0 = Dt[r * 3], d1 = Dt[r * 3 + 1], d2 = Dt[r * 3 + 2];
    T[r * 6 + 0] = d0;
    T[r * 6 + 1] = d1;
    T[r * 6 + 2] = d2;
    T[r * 6 + 3] = d1 * -rb.z + d2 * rb.y;
    T[r * 6 + 4] = d0 * rb.z + d2 * -rb.x;
    T[r * 6 + 5] = d0 * -rb.y + d1 * rb.x;
  }
  for (int r = 0; r < 3; ++r) {
    T[(3 + r) * 6 + 0] = 0.0;
    T[(3 + r) * 6 + 1] = 0.0;
    T[(3 + r) * 6 + 2] = 0.0;
    T[(3 + r) * 6 + 3] = Dr[r * 3];
    T[(3 + r) * 6 + 4] = Dr[r * 3 + 1];
    T[(3 + r) * 6 + 5] = Dr[r * 3 + 2];
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 6; ++c) C[r * 6 + c] += s * T[r * 6 + c];
  for (int c = 0; c < 6; ++c) {
    const double t0 = T[c], t1 = T[6 + c], t2 = T[12 + c];
    C[18 + c] += s * ((-ra.z * t1 + ra.y * t2) + T[18 + c]);
    C[24 + c] += s * ((ra.z * t0 + -ra.x * t2) + T[24 + c]);
    C[30 + c] += s * ((-ra.y * t0 + ra.x * t1) + T[30 + c]);
  }
}

// blk6::inv6 (amg.cpp:105-135): Gauss-Jordan with partial pivoting; false if singular.
SVXG_HD bool inv6(const double* A, double* Ainv) {
  double M[6][12];
  double scale = 0.0;
  for (int r = 0; r < 6; ++r) {
    for (int c = 0; c < 6; ++c) {
      M[r][c] = A[r * 6 + c];
      scale = maxd(scale, fabs(M[r][c]));
    }
    for (int c = 0; c < 6; ++c) M[r][6 + c] = (r == c) ? 1.0 : 0.0;
  }
  if (scale == 0.0) return false;
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    for (int r = c + 1; r < 6; ++r)
      if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
    if (fabs(M[piv][c]) <= 1e-15 * scale) return false;
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
  return true;
}

// Amg::finalize's diagonal inverse with its regularised retry (amg.cpp:231-243).
SVXG_HD bool inv6_regularised(const double* D, double* Dinv) {
  if (inv6(D, Dinv)) return true;
  double Dr[36];
  for (int q = 0; q < 36; ++q) Dr[q] = D[q];
  double tr = 0.0;
  for (int q = 0; q < 6; ++q) tr += fabs(Dr[q * 7]);
  const double eps = tr > 0 ? 1e-9 * tr : 1.0;
  for (int q = 0; q < 6; ++q) Dr[q * 7] += eps;
  return inv6(Dr, Dinv);
}

// blk6::fro6 (amg.cpp:137-141)
SVXG_HD double fro6(const double* M) {
  double s = 0.0;
  for (int i = 0; i < 36; ++i) s += M[i] * M[i];
  return sqrt(s);
}

// blk6::mv6 (amg.hpp:132-138): y = M x
SVXG_HD void mv6(const double* M, const double* x, double* y) {
  const double x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3], x4 = x[4], x5 = x[5];
  for (int r = 0; r < 6; ++r) {
    const double* m = M + r * 6;
    y[r] = m[0] * x0 + m[1] * x1 + m[2] * x2 + m[3] * x3 + m[4] * x4 + m[5] * x5;
  }
}

// mul6 (amg.cpp:59-67): C = A B
SVXG_HD void mul6(const double* A, const double* B, double* C) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int q = 0; q < 6; ++q) s += A[r * 6 + q] * B[q * 6 + c];
      C[r * 6 + c] = s;
    }
}

// mul6_add<trans> (amg.cpp:69-78): C += A B (A^T B if trans)
template <bool trans>
SVXG_HD void mul6_add(const double* A, const double* B, double* C) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int q = 0; q < 6; ++q) s += (trans ? A[q * 6 + r] : A[r * 6 + q]) * B[q * 6 + c];
      C[r * 6 + c] = C[r * 6 + c] + s;
    }
}

// bond_strength (stress.cpp:14-21): ft, fb, fc, cohesion, friction of the weaker side (or the
// bond's own section), scaled by strength / fragility
SVXG_HD void bond_strength(const svxg_bond& b, double fragility, const svxg_material* mats, double* S) {
  const double s = b.strength / maxd(1e-6, fragility);
  if (b.sectioned) {
    S[0] = s * (double)b.ft;
    S[1] = s * (double)b.fb;
    S[2] = s * (double)b.fc;
    S[3] = s * (double)b.coh;
    S[4] = (double)b.mu;
  } else {
    const svxg_material& A = mats[b.ma];
    const svxg_material& B = mats[b.mb];
    S[0] = s * mind(A.ft, B.ft);
    S[1] = s * mind(A.fb, B.fb);
    S[2] = s * mind(A.fc, B.fc);
    S[3] = s * mind(A.cohesion, B.cohesion);
    S[4] = mind(A.friction, B.friction);
  }
}

// bond_utilization (stress.cpp:23-57); mode: SVXG_FAIL_*
SVXG_HD double bond_utilization(const svxg_bond& b, const svxg_bond_load& L, double fragility,
                                const svxg_material* mats, uint8_t* mode) {
  double S[5];
  bond_strength(b, fragility, mats, S);
  const double kWeakest = 1e-9;
  S[0] = maxd(S[0], kWeakest);
  S[1] = maxd(S[1], kWeakest);
  S[2] = maxd(S[2], kWeakest);
  const double Ar = maxd(b.area, 1e-12);
  const double sN = L.N / Ar;
  const double sb = (b.s2 > 0 ? fabs(L.M1) * b.c2 / b.s2 : 0.0) + (b.s1 > 0 ? fabs(L.M2) * b.c1 / b.s1 : 0.0);
  double phi_t;
  if (sN >= 0.0) {
    phi_t = sN / S[0] + sb / S[1];
  } else {
    phi_t = maxd(0.0, sb + sN) / S[1];
  }
  const double phi_c = maxd(0.0, sb - sN) / S[2];
  const double J = maxd(b.s1 + b.s2, 1e-18);
  const double tau = 1.5 * sqrt(L.V1 * L.V1 + L.V2 * L.V2) / Ar + fabs(L.T) * b.rmax / J;
  const double cap = maxd(S[3] + S[4] * maxd(0.0, -sN), kWeakest);
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
  *mode = phi > 0 ? m : (uint8_t)SVXG_FAIL_NONE;
  return phi;
}

// StressProblem::bond_load (stress.cpp:477-502) from the two nodes' displacements (null: fixed
// or a support).
SVXG_HD svxg_bond_load bond_load(const svxg_bond& b, const svxg_material* mats, V3d ca, const double* ua, V3d cb,
                                 const double* ub) {
  const svxg_material& A = mats[b.ma];
  const svxg_material& B = mats[b.mb];
  double Ba[36], Bb[36];
  double xa[6] = {0, 0, 0, 0, 0, 0}, xb[6] = {0, 0, 0, 0, 0, 0};
  rigid_block(sub3(v3of(b.p), ca), Ba);
  if (ua) mv6(Ba, ua, xa);
  if (b.b >= 0) {
    rigid_block(sub3(v3of(b.p), cb), Bb);
    if (ub) mv6(Bb, ub, xb);
  }
  const V3d dt = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
  const V3d dr = {xb[3] - xa[3], xb[4] - xa[4], xb[5] - xa[5]};
  const double la = maxd(b.la, 1e-4), lb = maxd(b.lb, 1e-4);
  const double invE = la / A.E + lb / B.E;
  const double invG = la / A.G + lb / B.G;
  svxg_bond_load L;
  L.N = b.area / invE * dot3(dt, v3of(b.n));
  L.V1 = (5.0 / 6.0) * b.area / invG * dot3(dt, v3of(b.t1));
  L.V2 = (5.0 / 6.0) * b.area / invG * dot3(dt, v3of(b.t2));
  L.T = 0.8 * (b.s1 + b.s2) / invG * dot3(dr, v3of(b.n));
  L.M1 = b.s2 / invE * dot3(dr, v3of(b.t1));
  L.M2 = b.s1 / invE * dot3(dr, v3of(b.t2));
  return L;
}

}  // namespace svxg
