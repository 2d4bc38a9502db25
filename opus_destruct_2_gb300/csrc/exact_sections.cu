// exact_sections.cu - the bonds of voxel-face interfaces on the device: the world's section
// geometry, SecAcc::finish_lattice / finish_general (core/src/world/world_internal.hpp:133-352),
// and section_strengths / section_strengths_general (world_internal.hpp:370-441), as World::Impl
// builds a structure's bonds
// (core/src/world/world.cpp:839-850). One thread per bond walks its faces in order (each sum in
// the reference's order; compiled with -fmad=false), so every field equals the reference's.
//
// Per bond: the interface normal (the mean face normal from a to b; a support's face axis), its
// frame (frame_of), the faces' projected weights and centroid, the principal axes of the
// section (the eigenvector of the 2x2 second-moment matrix, sqrt only), area, s1/s2 with each
// face's own inertia, c1/c2/rmax, the spring lengths la/lb, the strength multiplier, and the
// section strengths (each face as strong as the weaker of its two voxels' materials times the
// condition of the more damaged, averaged).
#include "blk6.cuh"
#include "problem.cuh"

namespace svxg {
namespace {

constexpr int kT = 128;

__device__ __forceinline__ double comp(V3d a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ void add_comp(V3d& a, int i, double v) {
  if (i == 0) a.x += v;
  else if (i == 1) a.y += v;
  else a.z += v;
}
__device__ __forceinline__ V3d scale3(V3d a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3d cross3(V3d a, V3d b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3d normalized3(V3d a) {  // vec.hpp:47-50
  const double n = sqrt(dot3(a, a));
  return n > 0 ? scale3(a, 1.0 / n) : V3d{0, 0, 0};
}
__device__ __forceinline__ void frame_of(V3d n, V3d& t1, V3d& t2) {  // world_internal.hpp:64-69
  const double ax = fabs(n.x), ay = fabs(n.y), az = fabs(n.z);
  const V3d e = (ax <= ay && ax <= az) ? V3d{1, 0, 0} : (ay <= az ? V3d{0, 1, 0} : V3d{0, 0, 1});
  t1 = normalized3(cross3(n, e));
  t2 = cross3(n, t1);
}
__device__ __forceinline__ V3d face_centre(const svxg_face& F, double h) {
  V3d x = {h * F.x, h * F.y, h * F.z};
  add_comp(x, F.axis, 0.5 * h);
  return x;
}
__device__ __forceinline__ const svxg_material& side_material(const svxg_material* mats, uint8_t a, uint8_t b) {
  const int id = (a != 0 ? (a & 0x7F) : (b & 0x7F)) - 1;  // (air takes the other side's material)
  return mats[id >= 0 && id < SVXG_MAX_MATERIALS ? id : 0];
}

__device__ __forceinline__ V3d xf_dir(const svxg_lattice* X, V3d d) {  // LatticeXf::dir_to, M3 * V3
  if (!X || X->identity) return d;
  const double* R = X->R;
  return {R[0] * d.x + R[1] * d.y + R[2] * d.z, R[3] * d.x + R[4] * d.y + R[5] * d.z,
          R[6] * d.x + R[7] * d.y + R[8] * d.z};
}
__device__ __forceinline__ V3d xf_to(const svxg_lattice* X, V3d s) {  // LatticeXf::to
  if (!X || X->identity) return s;
  const V3d r = xf_dir(X, s);
  return {X->off[0] + r.x, X->off[1] + r.y, X->off[2] + r.z};
}

// element k of a general section (faces first, then junction samples): its point, normal, area
// and side (finish_general, world_internal.hpp:246-272)
struct Elem {
  V3d x, n;
  double ar, sd;
};
__device__ __forceinline__ Elem general_elem(int32_t k, int32_t nf, const svxg_face* F, const svxg_junction* J,
                                             const svxg_lattice* X, const svxg_lattice* lats, int32_t samples,
                                             double h) {
  Elem e;
  if (k < nf) {
    const svxg_face Fa = F[k];
    e.x = xf_to(X, face_centre(Fa, h));
    V3d n0 = {0, 0, 0};
    add_comp(n0, Fa.axis, double(Fa.sign));
    e.n = xf_dir(X, n0);
    e.ar = h * h;
    e.sd = h;
    return e;
  }
  const svxg_junction s = J[k - nf];
  const svxg_lattice* Xs = &lats[s.vg];
  const double hs = Xs->h, sj = hs / double(samples > 1 ? samples : 1);
  const int a = s.face >> 1, a1 = (a + 1) % 3, a2 = (a + 2) % 3;
  const double sg = (s.face & 1) ? 1.0 : -1.0;
  const int i = s.sub / samples, j = s.sub % samples;
  V3d p = {hs * s.v[0], hs * s.v[1], hs * s.v[2]};
  add_comp(p, a, sg * (0.5 * hs + 0.0));
  add_comp(p, a1, ((i + 0.5) / double(samples) - 0.5) * hs);
  add_comp(p, a2, ((j + 0.5) / double(samples) - 0.5) * hs);
  e.x = xf_to(Xs, p);
  V3d fn = {0, 0, 0};
  add_comp(fn, a, sg);
  e.n = scale3(xf_dir(Xs, fn), double(s.sign));
  e.ar = sj * sj * double(s.weight);
  e.sd = sj;
  return e;
}

// SecAcc::finish_general (world_internal.hpp:237-352) + section_strengths_general (:404-441)
__device__ void finish_general(const svxg_section& S, const svxg_face* F, const svxg_junction* J,
                               const svxg_lattice* lats, int32_t samples, const svxg_node* nodes,
                               const svxg_material* mats, svxg_bond& B) {
  const int32_t nf = S.faces, nj = S.junctions, ne = nf + nj;
  B.faces = ne;
  const double h = S.h;
  const svxg_lattice* X = lats ? &lats[S.grid] : nullptr;
  double atot = 0.0;
  for (int32_t k = 0; k < ne; ++k) atot += general_elem(k, nf, F, J, X, lats, samples, h).ar;
  const V3d ca = v3of(nodes[S.a].c);
  const bool has_b = S.b >= 0;
  const V3d cb = has_b ? v3of(nodes[S.b].c) : ca;
  V3d n = {0, 0, 0};
  if (has_b || nj) {
    for (int32_t k = 0; k < ne; ++k) {
      const Elem e = general_elem(k, nf, F, J, X, lats, samples, h);
      const V3d t = scale3(e.n, e.ar);
      n.x += t.x;
      n.y += t.y;
      n.z += t.z;
    }
    const double tiny = 1e-12 * atot * atot;
    if (dot3(n, n) <= tiny && has_b) n = sub3(cb, ca);
    if (dot3(n, n) <= tiny) n = V3d{0, 0, 1};
    n = normalized3(n);
  } else {
    V3d e = {0, 0, 0};
    add_comp(e, S.axis, double(S.sign));
    n = xf_dir(X, e);
  }
  V3d t1, t2;
  frame_of(n, t1, t2);
  double W = 0.0;
  V3d pc = {0, 0, 0};
  for (int32_t k = 0; k < ne; ++k) {
    const Elem e = general_elem(k, nf, F, J, X, lats, samples, h);
    const double w = e.ar * maxd(0.05, fabs(dot3(n, e.n)));
    W += w;
    pc.x += e.x.x * w;
    pc.y += e.x.y * w;
    pc.z += e.x.z * w;
  }
  pc = scale3(pc, 1.0 / W);
  {
    double s11 = 0.0, s22 = 0.0, s12 = 0.0;
    for (int32_t k = 0; k < ne; ++k) {
      const Elem e = general_elem(k, nf, F, J, X, lats, samples, h);
      const double w = e.ar * maxd(0.05, fabs(dot3(n, e.n)));
      const V3d d = sub3(e.x, pc);
      const double y1 = dot3(d, t1), y2 = dot3(d, t2);
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
        const V3d u1 = {t1.x * e1 + t2.x * e2, t1.y * e1 + t2.y * e2, t1.z * e1 + t2.z * e2};
        const V3d u2 = {t2.x * e1 - t1.x * e2, t2.y * e1 - t1.y * e2, t2.z * e1 - t1.z * e2};
        t1 = u1;
        t2 = u2;
      }
    }
  }
  B.n = {n.x, n.y, n.z};
  B.t1 = {t1.x, t1.y, t1.z};
  B.t2 = {t2.x, t2.y, t2.z};
  B.p = {pc.x, pc.y, pc.z};
  B.area = maxd(W, 0.25 * atot);
  double s1 = 0.0, s2 = 0.0, m1 = 0.0, m2 = 0.0, own = 0.0;
  for (int32_t k = 0; k < ne; ++k) {
    const Elem e = general_elem(k, nf, F, J, X, lats, samples, h);
    const double w = e.ar * maxd(0.05, fabs(dot3(n, e.n)));
    const V3d d = sub3(e.x, pc);
    const double y1 = dot3(d, t1), y2 = dot3(d, t2);
    s1 += w * y1 * y1;
    s2 += w * y2 * y2;
    m1 = maxd(m1, fabs(y1) + 0.5 * e.sd);
    m2 = maxd(m2, fabs(y2) + 0.5 * e.sd);
    own += w * e.sd * e.sd;
  }
  own /= W;
  B.s1 = s1 + B.area * own / 12.0;
  B.s2 = s2 + B.area * own / 12.0;
  B.c1 = m1;
  B.c2 = m2;
  B.rmax = sqrt(B.c1 * B.c1 + B.c2 * B.c2);
  if (has_b) {
    const V3d d = sub3(cb, ca);
    const double L = maxd(maxd(fabs(dot3(d, n)), 0.5 * sqrt(dot3(d, d))), 0.5 * h);
    const double x = dot3(sub3(pc, ca), n), lo = 0.1 * L, hi = 0.9 * L;
    B.la = x < lo ? lo : (hi < x ? hi : x);
    B.lb = L - B.la;
  } else {
    B.la = maxd(0.25 * h, dot3(sub3(pc, ca), n));
    B.lb = 0.5 * h;
  }
  B.strength = mind(S.strength_a, S.strength_b);
  if (S.sectioned) {
    double ft = 0, fb = 0, fc = 0, coh = 0, mu = 0, wsum = 0;
    const double sw = 1.0 / double(samples * samples > 1 ? samples * samples : 1);
    for (int32_t k = 0; k < ne; ++k) {
      uint8_t va, vb, da, db;
      double w;
      if (k < nf) {
        va = F[k].vox_lo;
        vb = F[k].vox_hi;
        da = F[k].damage_lo;
        db = F[k].damage_hi;
        w = 1.0;
      } else {
        const svxg_junction& s = J[k - nf];
        va = s.vox_v;
        da = s.damage_v;
        vb = s.kind == 1 ? va : s.vox_o;  // (a sample into the unknown world: its own voxel)
        db = s.kind == 1 ? da : s.damage_o;
        w = sw * double(1.0f);
      }
      const svxg_material& A = side_material(mats, va, vb);
      const svxg_material& M = side_material(mats, vb, va);
      const int dm = da > db ? da : db;
      const double cond = maxd(1e-6, 1.0 - double(dm) / 255.0);
      ft += w * cond * mind(A.ft, M.ft);
      fb += w * cond * mind(A.fb, M.fb);
      fc += w * cond * mind(A.fc, M.fc);
      coh += w * cond * mind(A.cohesion, M.cohesion);
      mu += w * mind(A.friction, M.friction);
      wsum += w;
    }
    if (ne > 0 && wsum > 0.0) {
      const double w = 1.0 / wsum;
      B.sectioned = 1;
      B.ft = float(ft * w);
      B.fb = float(fb * w);
      B.fc = float(fc * w);
      B.coh = float(coh * w);
      B.mu = float(mu * w);
    }
  }
}

__global__ void k_build_bonds(int32_t nb, int32_t n_nodes, int64_t n_faces, int64_t n_juncs, int32_t n_lats,
                              int32_t samples, const svxg_node* __restrict__ nodes,
                              const svxg_section* __restrict__ secs, const svxg_face* __restrict__ faces,
                              const svxg_junction* __restrict__ juncs, const svxg_lattice* __restrict__ lats,
                              const svxg_material* __restrict__ mats, svxg_bond* __restrict__ out, int32_t* bad) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const svxg_section S = secs[k];
  svxg_bond B;
  memset(&B, 0, sizeof(B));
  // (a section whose nodes, faces, samples or lattices lie outside the arrays: a broken, empty
  // bond, counted)
  bool ok = S.a >= 0 && S.a < n_nodes && S.b < n_nodes && S.faces >= 0 && S.first_face >= 0 &&
            S.first_face + S.faces <= n_faces && (S.b >= 0 || S.axis <= 2) && S.junctions >= 0 &&
            (S.junctions == 0 || (S.first_junction >= 0 && S.first_junction + S.junctions <= n_juncs)) &&
            (n_lats == 0 ? S.junctions == 0 : int32_t(S.grid) < n_lats) && samples >= 1;
  for (int32_t f = 0; ok && f < S.faces; ++f) ok = faces[S.first_face + f].axis <= 2;
  for (int32_t j = 0; ok && j < S.junctions; ++j) {
    const svxg_junction& J = juncs[S.first_junction + j];
    ok = J.vg < n_lats && J.face < 6;
  }
  if (!ok) {
    B.a = S.a;
    B.b = S.b;
    B.broken = 1;
    B.tag = k;
    out[k] = B;
    if (bad) atomicAdd(bad, 1);
    return;
  }
  const svxg_face* F = faces + S.first_face;
  const int32_t nf = S.faces;
  if (S.junctions > 0 || (n_lats > 0 && !lats[S.grid].identity)) {  // SecAcc::finish (world_internal.hpp:130-133)
    B.a = S.a;
    B.b = S.b;
    B.ma = S.ma;
    B.mb = S.mb;
    finish_general(S, F, juncs + S.first_junction, n_lats > 0 ? lats : nullptr, samples, nodes, mats, B);
    B.tag = k;
    out[k] = B;
    return;
  }
  B.a = S.a;
  B.b = S.b;
  B.ma = S.ma;
  B.mb = S.mb;
  B.faces = nf;
  const double h = S.h, A1 = h * h;
  const V3d ca = v3of(nodes[S.a].c);
  const bool has_b = S.b >= 0;
  const V3d cb = has_b ? v3of(nodes[S.b].c) : ca;
  V3d n = {0, 0, 0};
  if (has_b) {
    for (int32_t f = 0; f < nf; ++f) add_comp(n, F[f].axis, double(F[f].sign));
    if (dot3(n, n) < 1e-12) n = sub3(cb, ca);
    if (dot3(n, n) < 1e-12) n = V3d{0, 0, 1};
    n = normalized3(n);
  } else {
    add_comp(n, S.axis, double(S.sign));
  }
  V3d t1, t2;
  frame_of(n, t1, t2);
  double W = 0.0;
  V3d pc = {0, 0, 0};
  for (int32_t f = 0; f < nf; ++f) {
    const svxg_face Fa = F[f];
    const V3d x = face_centre(Fa, h);
    const double w = A1 * maxd(0.05, fabs(comp(n, Fa.axis)));
    W += w;
    pc.x += x.x * w;
    pc.y += x.y * w;
    pc.z += x.z * w;
  }
  pc = scale3(pc, 1.0 / W);
  {
    double s11 = 0.0, s22 = 0.0, s12 = 0.0;
    for (int32_t f = 0; f < nf; ++f) {
      const svxg_face Fa = F[f];
      const V3d d = sub3(face_centre(Fa, h), pc);
      const double w = A1 * maxd(0.05, fabs(comp(n, Fa.axis)));
      const double y1 = dot3(d, t1), y2 = dot3(d, t2);
      s11 += w * y1 * y1;
      s22 += w * y2 * y2;
      s12 += w * y1 * y2;
    }
    if (fabs(s12) > 1e-9 * (s11 + s22)) {
      const double half = 0.5 * (s11 - s22);
      const double l1 = 0.5 * (s11 + s22) + sqrt(half * half + s12 * s12);
      double e1 = s12, e2 = l1 - s11;  // (the better conditioned of the two forms)
      if (fabs(l1 - s22) > fabs(e2)) {
        e1 = l1 - s22;
        e2 = s12;
      }
      const double en = sqrt(e1 * e1 + e2 * e2);
      if (en > 0.0) {
        e1 /= en;
        e2 /= en;
        const V3d u1 = {t1.x * e1 + t2.x * e2, t1.y * e1 + t2.y * e2, t1.z * e1 + t2.z * e2};
        const V3d u2 = {t2.x * e1 - t1.x * e2, t2.y * e1 - t1.y * e2, t2.z * e1 - t1.z * e2};
        t1 = u1;
        t2 = u2;
      }
    }
  }
  B.n = {n.x, n.y, n.z};
  B.t1 = {t1.x, t1.y, t1.z};
  B.t2 = {t2.x, t2.y, t2.z};
  B.p = {pc.x, pc.y, pc.z};
  B.area = maxd(W, 0.25 * nf * A1);
  double s1 = 0.0, s2 = 0.0, m1 = 0.0, m2 = 0.0;
  for (int32_t f = 0; f < nf; ++f) {
    const svxg_face Fa = F[f];
    const V3d d = sub3(face_centre(Fa, h), pc);
    const double w = A1 * maxd(0.05, fabs(comp(n, Fa.axis)));
    const double y1 = dot3(d, t1), y2 = dot3(d, t2);
    s1 += w * y1 * y1;
    s2 += w * y2 * y2;
    m1 = maxd(m1, fabs(y1));
    m2 = maxd(m2, fabs(y2));
  }
  B.s1 = s1 + B.area * A1 / 12.0;
  B.s2 = s2 + B.area * A1 / 12.0;
  B.c1 = m1 + 0.5 * h;
  B.c2 = m2 + 0.5 * h;
  B.rmax = sqrt(B.c1 * B.c1 + B.c2 * B.c2);
  if (has_b) {
    const V3d d = sub3(cb, ca);
    const double L = maxd(maxd(fabs(dot3(d, n)), 0.5 * sqrt(dot3(d, d))), 0.5 * h);
    const double x = dot3(sub3(pc, ca), n), lo = 0.1 * L, hi = 0.9 * L;
    B.la = x < lo ? lo : (hi < x ? hi : x);  // std::clamp
    B.lb = L - B.la;
  } else {
    B.la = maxd(0.25 * h, dot3(sub3(pc, ca), n));
    B.lb = 0.5 * h;
  }
  B.strength = mind(S.strength_a, S.strength_b);
  if (S.sectioned && nf > 0) {
    double ft = 0, fb = 0, fc = 0, coh = 0, mu = 0;
    for (int32_t f = 0; f < nf; ++f) {
      const svxg_face Fa = F[f];
      const svxg_material& A = side_material(mats, Fa.vox_lo, Fa.vox_hi);
      const svxg_material& M = side_material(mats, Fa.vox_hi, Fa.vox_lo);
      const int dm = Fa.damage_lo > Fa.damage_hi ? Fa.damage_lo : Fa.damage_hi;
      const double cond = maxd(1e-6, 1.0 - double(dm) / 255.0);
      ft += cond * mind(A.ft, M.ft);
      fb += cond * mind(A.fb, M.fb);
      fc += cond * mind(A.fc, M.fc);
      coh += cond * mind(A.cohesion, M.cohesion);
      mu += mind(A.friction, M.friction);
    }
    const double w = 1.0 / double(nf);
    B.sectioned = 1;
    B.ft = float(ft * w);
    B.fb = float(fb * w);
    B.fc = float(fc * w);
    B.coh = float(coh * w);
    B.mu = float(mu * w);
  }
  B.tag = k;
  out[k] = B;
}

}  // namespace

int build_bonds_device(const svxg_node* nodes, int32_t n, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                       int64_t nf, const svxg_junction* juncs, int64_t nj, const svxg_lattice* lats, int32_t nl,
                       int32_t samples, const svxg_material* mats, svxg_bond* out, int32_t* bad, cudaStream_t st) {
  if (nb <= 0) return SVXG_OK;
  (k_build_bonds<<<unsigned((nb + kT - 1) / kT), kT, 0, st>>>(nb, n, nf, nj, nl, samples, nodes, secs, faces, juncs,
                                                             lats, mats, out, bad), SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

}  // namespace svxg
