// exact_sections.cu - the bonds of voxel-face interfaces on the device: the world's section
// geometry, SecAcc::finish_lattice (core/src/world/world_internal.hpp:133-232), and
// section_strengths (world_internal.hpp:370-399), as World::Impl builds a structure's bonds
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

__global__ void k_build_bonds(int32_t nb, int32_t n_nodes, int64_t n_faces, const svxg_node* __restrict__ nodes,
                              const svxg_section* __restrict__ secs, const svxg_face* __restrict__ faces,
                              const svxg_material* __restrict__ mats, svxg_bond* __restrict__ out, int32_t* bad) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const svxg_section S = secs[k];
  svxg_bond B;
  memset(&B, 0, sizeof(B));
  // (a section whose nodes or faces lie outside the arrays: a broken, empty bond, counted)
  bool ok = S.a >= 0 && S.a < n_nodes && S.b < n_nodes && S.faces >= 0 && S.first_face >= 0 &&
            S.first_face + S.faces <= n_faces && (S.b >= 0 || S.axis <= 2);
  for (int32_t f = 0; ok && f < S.faces; ++f) ok = faces[S.first_face + f].axis <= 2;
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
                       int64_t nf, const svxg_material* mats, svxg_bond* out, int32_t* bad, cudaStream_t st) {
  if (nb <= 0) return SVXG_OK;
  (k_build_bonds<<<unsigned((nb + kT - 1) / kT), kT, 0, st>>>(nb, n, nf, nodes, secs, faces, mats, out, bad),
   SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  return SVXG_OK;
}

}  // namespace svxg
