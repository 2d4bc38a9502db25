// host_loads.cpp - the loads a caller builds before a solve, and the reference's free judge
// functions, on the host (built without FP contraction, like the reference: the same bits on x86
// and Arm as the reference's own arithmetic in the same order).
//
//   svxg_structure_loads  World::Impl::load_vector (core/src/world/world.cpp:966-974)
//   svxg_pin_reference    pin_reference (core/src/world/world_pieces.cpp:313-326)
//   svxg_body_loads       World::Impl::body_stress_run's loads (world_pieces.cpp:566-603): inertial
//                         relief of a moving piece and its point forces through add_force
//   svxg_bond_strength / svxg_bond_utilization  bond_strength / bond_utilization
//                         (core/src/stress/stress.cpp:14-57), from the same source as the device judge
#include <cmath>
#include <cstring>

#include "blk6.cuh"
#include "svxg.h"

namespace {

struct Vh {
  double x, y, z;
};
Vh vh(const svxg_v3& a) { return {a.x, a.y, a.z}; }
Vh add(Vh a, Vh b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
Vh sub(Vh a, Vh b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
Vh scale(Vh a, double s) { return {a.x * s, a.y * s, a.z * s}; }
Vh cross(Vh a, Vh b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dot(Vh a, Vh b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// a 3x3 row-major matrix times a vector, and times a matrix (base/vec.hpp:63-72)
Vh mv(const double* A, Vh v) {
  return {A[0] * v.x + A[1] * v.y + A[2] * v.z, A[3] * v.x + A[4] * v.y + A[5] * v.z,
          A[6] * v.x + A[7] * v.y + A[8] * v.z};
}
void mm(const double* A, const double* B, double* R) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
}
void transpose(const double* A, double* R) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = A[3 * c + r];
}

// the rotation of a unit quaternion (x, y, z, w) as a matrix (base/vec.hpp:111-120)
void to_matrix(const double* q, double* R) {
  const double xx = q[0] * q[0], yy = q[1] * q[1], zz = q[2] * q[2];
  const double xy = q[0] * q[1], xz = q[0] * q[2], yz = q[1] * q[2];
  const double wx = q[3] * q[0], wy = q[3] * q[1], wz = q[3] * q[2];
  const double m[9] = {1 - 2 * (yy + zz), 2 * (xy - wz),     2 * (xz + wy),
                       2 * (xy + wz),     1 - 2 * (xx + zz), 2 * (yz - wx),
                       2 * (xz - wy),     2 * (yz + wx),     1 - 2 * (xx + yy)};
  std::memcpy(R, m, sizeof(m));
}

// v rotated by the conjugate of q (base/vec.hpp:103-109): the world-to-shape rotation
Vh rotate_inv(const double* q, Vh v) {
  const Vh u{-q[0], -q[1], -q[2]};
  const Vh t = scale(cross(u, v), 2.0);
  return add(add(v, scale(t, q[3])), cross(u, t));
}

// StressProblem::add_force (core/src/stress/stress.cpp:504-514): a force F at point `at` on a node
// with centre c
void add_force(double* f, int32_t node, Vh c, Vh F, Vh at) {
  double* fi = f + 6 * int64_t(node);
  fi[0] += F.x;
  fi[1] += F.y;
  fi[2] += F.z;
  const Vh r = sub(at, c);
  const Vh m = cross(r, F);
  fi[3] += m.x;
  fi[4] += m.y;
  fi[5] += m.z;
}

}  // namespace

extern "C" {

int svxg_structure_loads(int32_t n, const double* weight, const double* ext, double* f) {
  if (n < 0 || (n > 0 && (!weight || !f))) return SVXG_ERR_ARG;
  for (int64_t i = 0; i < n; ++i) {
    double* fi = f + 6 * i;
    for (int q = 0; q < 6; ++q) fi[q] = 0.0;
    fi[2] = -weight[i];
    // (a missing ext adds zeros, as the world's zero-filled ext_solved does: -0.0 + 0.0 is +0.0)
    for (int q = 0; q < 6; ++q) fi[q] += ext ? ext[6 * i + q] : 0.0;
  }
  return SVXG_OK;
}

int32_t svxg_pin_reference(svxg_node* nodes, int32_t n, svxg_v3 com) {
  if (n <= 0 || !nodes) return -1;
  int32_t pin = 0;
  double best = 1e300;
  const Vh cm = vh(com);
  for (int32_t i = 0; i < n; ++i) {
    nodes[i].fixed = 0;
    const Vh d = sub(vh(nodes[i].c), cm);
    const double d2 = dot(d, d);
    if (d2 < best) {
      best = d2;
      pin = i;
    }
  }
  nodes[pin].fixed = 1;
  return pin;
}

int svxg_body_loads(const svxg_body_state* b, const svxg_node* nodes, int32_t n, const svxg_v3* node_com,
                    const double* node_mass, const double* node_inertia, const svxg_point_force* forces,
                    int32_t nforces, int32_t inertia, double* f) {
  if (!b || n < 0 || nforces < 0 || (n > 0 && (!nodes || !f)) || (nforces > 0 && !forces) ||
      (inertia && n > 0 && (!node_com || !node_mass || !node_inertia)))
    return SVXG_ERR_ARG;
  for (int64_t k = 0; k < 6 * int64_t(n); ++k) f[k] = 0.0;
  double R[9], Rt[9];
  to_matrix(b->q, R);
  transpose(R, Rt);
  const Vh g{0, 0, -b->gravity};
  const Vh x = vh(b->x), com = vh(b->com), w = vh(b->w);
  if (inertia) {
    Vh Ft{0, 0, 0}, tau{0, 0, 0};
    for (int32_t k = 0; k < nforces; ++k) {
      const Vh F = vh(forces[k].F);
      Ft = add(Ft, F);
      tau = add(tau, cross(sub(vh(forces[k].p), x), F));
    }
    double T[9], Iw[9], Iwi[9];
    mm(R, b->inertia, T);
    mm(T, Rt, Iw);
    mm(R, b->inv_inertia, T);
    mm(T, Rt, Iwi);
    const Vh a = add(scale(Ft, b->inv_mass), g);
    const Vh alpha = mv(Iwi, sub(tau, cross(w, mv(Iw, w))));
    for (int32_t i = 0; i < n; ++i) {
      const Vh rw = mv(R, sub(vh(node_com[i]), com));
      const Vh ai = add(add(a, cross(alpha, rw)), cross(w, cross(w, rw)));
      const Vh Fi = mv(Rt, scale(sub(g, ai), node_mass[i]));
      double Ii[9];
      mm(R, node_inertia + 9 * int64_t(i), T);
      mm(T, Rt, Ii);
      const Vh Mi = mv(Rt, scale(add(mv(Ii, alpha), cross(w, mv(Ii, w))), -1.0));
      double* fi = f + 6 * int64_t(i);
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
    // (the force in the shape frame at its point in the shape frame, Body::to_shape, phys/rigid.hpp:206)
    const Vh at = add(com, rotate_inv(b->q, sub(vh(forces[k].p), x)));
    add_force(f, i, vh(nodes[i].c), mv(Rt, vh(forces[k].F)), at);
  }
  return SVXG_OK;
}

int svxg_bond_strength(const svxg_bond* b, double fragility, const svxg_material* mats, double* out) {
  if (!b || !mats || !out || b->ma >= SVXG_MAX_MATERIALS || b->mb >= SVXG_MAX_MATERIALS) return SVXG_ERR_ARG;
  svxg::bond_strength(*b, fragility, mats, out);
  return SVXG_OK;
}

double svxg_bond_utilization(const svxg_bond* b, const svxg_bond_load* L, double fragility, const svxg_material* mats,
                             uint8_t* mode) {
  uint8_t m = SVXG_FAIL_NONE;
  if (!b || !L || !mats || b->ma >= SVXG_MAX_MATERIALS || b->mb >= SVXG_MAX_MATERIALS) {
    if (mode) *mode = m;
    return -1.0;
  }
  const double phi = svxg::bond_utilization(*b, *L, fragility, mats, &m);
  if (mode) *mode = m;
  return phi;
}

}  // extern "C"
