// test_adapter.cpp - the C++20 host class (include/svxg_stress_problem.hpp) on the device, with the
// reference's own test cases written as the reference writes them (tests/core/test_stress.cpp).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

#include "svxg_stress_problem.hpp"

namespace {

int failures = 0;
#define CHECK(c)                                                        \
  do {                                                                  \
    if (!(c)) {                                                         \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);        \
      ++failures;                                                       \
    }                                                                   \
  } while (0)

bool approx(double a, double b, double eps) { return std::fabs(a - b) <= eps * std::fmax(std::fabs(a), std::fabs(b)); }

std::vector<svxg_material> materials() {
  // the presets the cases use: rc (id 0, also every unregistered id) and concrete (id 1)
  std::vector<svxg_material> m(SVXG_MAX_MATERIALS, svxg_material{30e9, 12.5e9, 2400, 1.2e6, 3.5e6, 30e6, 1.6e6, 0.7});
  m[1] = svxg_material{28e9, 11.5e9, 2300, 0.8e6, 1.2e6, 25e6, 1.2e6, 0.7};
  return m;
}

// test_stress.cpp:14-32
svxg_bond bond(const svxg::StressProblem& P, int32_t A, int32_t B, svxg_v3 n, svxg_v3 p, double a) {
  svxg_bond s{};
  s.a = A;
  s.b = B;
  s.ma = s.mb = 1;
  s.n = n;
  s.t1 = std::fabs(n.x) > 0.5 ? svxg_v3{0, 1, 0} : svxg_v3{1, 0, 0};
  s.t2 = {n.y * s.t1.z - n.z * s.t1.y, n.z * s.t1.x - n.x * s.t1.z, n.x * s.t1.y - n.y * s.t1.x};
  s.area = a * a;
  s.p = p;
  s.s1 = s.s2 = a * a * a * a / 12.0;
  s.c1 = s.c2 = 0.5 * a;
  s.rmax = std::sqrt(0.5) * a;
  const svxg_v3 ca = P.nodes[size_t(A)].c;
  s.la = std::fabs((p.x - ca.x) * n.x + (p.y - ca.y) * n.y + (p.z - ca.z) * n.z);
  if (B >= 0) {
    const svxg_v3 cb = P.nodes[size_t(B)].c;
    s.lb = std::fabs((cb.x - p.x) * n.x + (cb.y - p.y) * n.y + (cb.z - p.z) * n.z);
  } else {
    s.lb = s.la;
  }
  s.strength = 1.0;
  s.faces = 16;
  s.tag = -1;
  return s;
}

// test_stress.cpp:35-46
void cantilever(svxg::StressProblem& P, int n, double L, double mass) {
  P.mats = materials();
  for (int i = 0; i < n; ++i) {
    svxg_node nd{};
    nd.c = {(i + 0.5) * L, 0, 0};
    nd.mass = mass;
    P.nodes.push_back(nd);
  }
  P.bonds.push_back(bond(P, 0, -1, {-1, 0, 0}, {0, 0, 0}, L));
  for (int i = 0; i + 1 < n; ++i) P.bonds.push_back(bond(P, i, i + 1, {1, 0, 0}, {(i + 1) * L, 0, 0}, L));
}

std::vector<double> gravity(const svxg::StressProblem& P) {
  std::vector<double> f(6 * P.nodes.size(), 0.0);
  for (size_t i = 0; i < P.nodes.size(); ++i) f[6 * i + 2] = -9.81 * P.nodes[i].mass;
  return f;
}

// a grid of nx x ny x nz unit cells (0.5 m), face bonds between neighbours, supports under z = 0
void lattice(svxg::StressProblem& P, int nx, int ny, int nz) {
  P.mats = materials();
  const double h = 0.5;
  auto id = [&](int x, int y, int z) { return int32_t((z * ny + y) * nx + x); };
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        svxg_node nd{};
        nd.c = {(x + 0.5) * h, (y + 0.5) * h, (z + 0.5) * h};
        nd.mass = 300.0;
        P.nodes.push_back(nd);
      }
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const svxg_v3 c = P.nodes[size_t(id(x, y, z))].c;
        if (z == 0) P.bonds.push_back(bond(P, id(x, y, z), -1, {0, 0, -1}, {c.x, c.y, 0.0}, h));
        if (x + 1 < nx) P.bonds.push_back(bond(P, id(x, y, z), id(x + 1, y, z), {1, 0, 0}, {c.x + 0.5 * h, c.y, c.z}, h));
        if (y + 1 < ny) P.bonds.push_back(bond(P, id(x, y, z), id(x, y + 1, z), {0, 1, 0}, {c.x, c.y + 0.5 * h, c.z}, h));
        if (z + 1 < nz) P.bonds.push_back(bond(P, id(x, y, z), id(x, y, z + 1), {0, 0, 1}, {c.x, c.y, c.z + 0.5 * h}, h));
      }
}

bool same_load(const svxg_bond_load& a, const svxg_bond_load& b) {
  return a.N == b.N && a.V1 == b.V1 && a.V2 == b.V2 && a.T == b.T && a.M1 == b.M1 && a.M2 == b.M2;
}

double shear(const svxg_bond_load& L) { return std::sqrt(L.V1 * L.V1 + L.V2 * L.V2); }
double moment(const svxg_bond_load& L) { return std::sqrt(L.M1 * L.M1 + L.M2 * L.M2); }

}  // namespace

int main() {
  {  // test_stress.cpp:59-87: a cantilever carries its weight to the support (statics, exactly)
    const int n = 12;
    const double L = 0.5, m = 300.0;
    svxg::StressProblem P;
    cantilever(P, n, L, m);
    svxg_stress_options so = svxg_default_options();
    so.amg_min_nodes = 4;
    CHECK(P.assemble(so));
    std::vector<double> u;
    const svxg_pcg_result r = P.solve(gravity(P), u, 1e-10, 500, false);
    CHECK(r.converged);
    const svxg_bond_load root = P.bond_load(0, u);
    double W = 0.0, M = 0.0;
    for (int i = 0; i < n; ++i) {
      W += 9.81 * m;
      M += 9.81 * m * (i + 0.5) * L;
    }
    CHECK(approx(shear(root), W, 1e-6));
    CHECK(approx(moment(root), M, 1e-6));
    CHECK(std::fabs(root.N) < 1e-6 * W);
    const svxg_bond_load tip = P.bond_load(n - 1, u);
    CHECK(approx(shear(tip), 9.81 * m, 1e-6));
    CHECK(approx(moment(tip), 9.81 * m * 0.5 * L, 1e-6));
    const auto j = P.judge(1.0);
    CHECK(j.phi[0] > 50.0 * j.phi[size_t(n - 1)]);
  }
  {  // test_stress.cpp:154-174: removing a bond in place equals assembling without it
    svxg::StressProblem A, B;
    cantilever(A, 10, 0.5, 200.0);
    cantilever(B, 10, 0.5, 200.0);
    A.bonds.push_back(bond(A, 6, -1, {0, 0, -1}, {A.nodes[6].c.x, 0, -0.25}, 0.5));
    B.bonds.push_back(bond(B, 6, -1, {0, 0, -1}, {B.nodes[6].c.x, 0, -0.25}, 0.5));
    svxg_stress_options so = svxg_default_options();
    so.amg_min_nodes = 1 << 30;
    CHECK(A.assemble(so));
    A.remove_bond(3);
    B.bonds[3].broken = 1;
    CHECK(B.assemble(so));
    std::vector<double> ua, ub;
    A.solve(gravity(A), ua, 1e-11, 2000, false);
    B.solve(gravity(B), ub, 1e-11, 2000, false);
    double err = 0.0, mag = 0.0;
    for (size_t k = 0; k < ua.size(); ++k) {
      err = std::fmax(err, std::fabs(ua[k] - ub[k]));
      mag = std::fmax(mag, std::fabs(ub[k]));
    }
    CHECK(err <= 1e-6 * mag);
    CHECK(A.bonds[3].broken == 1 && A.bonds[3].in_k == 0);
  }
  {  // test_stress.cpp:293-305: no answer for non-finite loads, u = 0 for none
    svxg::StressProblem P;
    cantilever(P, 6, 0.5, 100.0);
    CHECK(P.assemble());
    std::vector<double> u(6 * P.nodes.size(), 1.0), f(6 * P.nodes.size(), 0.0);
    const svxg_pcg_result r0 = P.solve(f, u, 1e-9, 100, true);
    CHECK(r0.converged);
    for (double v : u) CHECK(v == 0.0);
    f[2] = NAN;
    const svxg_pcg_result r1 = P.solve(f, u, 1e-9, 100, false);
    CHECK(!r1.converged);
    CHECK(r1.breakdown);
  }
  {  // begin / iterate: the same conjugate-gradient sequence over several calls
    svxg::StressProblem P;
    cantilever(P, 40, 0.5, 100.0);
    svxg_stress_options so = svxg_default_options();
    so.amg_min_nodes = 1 << 30;
    CHECK(P.assemble(so));
    P.begin(gravity(P), {});
    int total = 0;
    svxg_pcg_result r{};
    for (int t = 0; t < 100 && !r.converged; ++t) {
      r = P.iterate(3, 1e-10);
      total += r.iters;
    }
    CHECK(r.converged);
    std::vector<double> u1, u2;
    P.current(u1);
    const svxg_pcg_result once = P.solve(gravity(P), u2, 1e-10, 1000, false);
    CHECK(once.iters == total);
    double err = 0.0, mag = 0.0;
    for (size_t k = 0; k < u1.size(); ++k) {
      err = std::fmax(err, std::fabs(u1[k] - u2[k]));
      mag = std::fmax(mag, std::fabs(u2[k]));
    }
    CHECK(err <= 1e-12 * mag);
  }
  {
    // the judge's break rounds: an overloaded cantilever breaks at its support, and the part that
    // no support holds retires (then nothing is left over strength)
    svxg::StressProblem P;
    cantilever(P, 8, 0.5, 2.0e5);
    CHECK(P.assemble());
    std::vector<double> u;
    svxg_cascade_options o = svxg_default_cascade_options();
    o.rtol = 1e-10;
    o.maxit = 1000;
    const auto c = P.cascade(gravity(P), u, o);
    CHECK(c.result.status == SVXG_CASCADE_SETTLED);
    CHECK(c.result.rounds >= 1 && !c.broken.empty() && c.broken[0] == 0);
    CHECK(int(c.retired.size()) == 8);
    CHECK(P.bonds[0].broken == 1);
    for (const svxg_node& nd : P.nodes) CHECK(nd.gone == 1);
  }
  {
    // a piece's break rounds on the same cantilever pinned at its root: rounds run, loads move
    svxg::StressProblem P;
    cantilever(P, 8, 0.5, 2.0e5);
    P.bonds.erase(P.bonds.begin());  // (no support: a free piece, pinned at node 0)
    P.nodes[0].fixed = 1;
    std::vector<double> f = gravity(P), u;
    svxg_piece_options o = svxg_default_piece_options();
    o.rtol = 1e-10;
    o.maxit = 1000;
    const auto r = P.piece_rounds(f, u, o);
    CHECK(r.result.checks >= 1);
    CHECK(r.broken.size() == r.modes.size());
    CHECK(r.result.status != SVXG_PIECE_SOLVE_FAILED && r.result.status != SVXG_PIECE_SINGULAR);
  }
  {
    // bonds from voxel faces: two voxels side by side (lattice voxel i centred at h i), one face
    std::vector<svxg_node> nodes(2);
    nodes[0].c = {0.0, 0.0, 0.0};
    nodes[1].c = {0.5, 0.0, 0.0};
    svxg_section sec{};
    sec.a = 0;
    sec.b = 1;
    sec.faces = 1;
    sec.sectioned = 1;
    sec.h = 0.5;
    sec.strength_a = sec.strength_b = 1.0;
    svxg_face fc{};
    fc.axis = 0;
    fc.sign = 1;
    fc.vox_lo = fc.vox_hi = 2;  // (material 1 on both sides)
    const auto b = svxg::build_bonds(nodes, {sec}, {fc}, materials());
    CHECK(b.size() == 1 && b[0].n.x == 1.0 && b[0].area == 0.25 && b[0].la == 0.25 && b[0].lb == 0.25);
    CHECK(b[0].sectioned == 1 && b[0].faces == 1);
  }
  {
    // the reference's callers ask bond_load bond by bond at one u (world.cpp:1174, :1927): over a
    // graph of about 10k bonds that is one device pass for the whole loop, the same numbers as the
    // every-bond pass, and a changed u at a bond's ends makes a new pass
    svxg::StressProblem P;
    lattice(P, 24, 24, 6);
    CHECK(P.bonds.size() > 10000);
    CHECK(P.assemble());
    std::vector<double> u;
    CHECK(P.solve(gravity(P), u, 1e-8, 500, false).converged);
    const auto all = P.bond_loads(u);
    CHECK(all.size() == P.bonds.size());
    const auto t0 = std::chrono::steady_clock::now();
    double sum = 0.0;
    bool equal = true;
    for (int32_t b = 0; b < int32_t(P.bonds.size()); ++b) {
      const svxg_bond_load L = P.bond_load(b, u);
      sum += std::fabs(L.N);
      equal = equal && same_load(L, all[size_t(b)]);
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    CHECK(equal);
    CHECK(P.bond_load_passes() == 1);
    std::printf("bond_load loop: %zu bonds, %lld device pass(es), %.3f ms (sum |N| %.6g)\n", P.bonds.size(),
                (long long)P.bond_load_passes(), ms, sum);
    std::vector<double> u2 = u;
    const svxg_bond& b0 = P.bonds[0];
    u2[6 * size_t(b0.a) + 2] *= 2.0;
    (void)P.bond_load(0, u2);
    CHECK(P.bond_load_passes() == 2);
    CHECK(same_load(P.bond_load(0, u2), P.bond_loads(u2)[0]));
    // stress.hpp:116-117: the solver's bytes are what release() frees; the graph stays
    const int64_t held = P.memory_bytes(), used = P.memory_bytes(svxg::Bytes::Used), solver = P.solver_bytes();
    CHECK(solver > 0 && solver < held && used <= held);
    P.release();
    CHECK(P.solver_bytes() < solver);
    CHECK(!P.assembled());
  }
  {
    // the reference's error contract (no exceptions): a wrong-sized load is no answer
    svxg::StressProblem P;
    cantilever(P, 6, 0.5, 100.0);
    CHECK(P.assemble());
    std::vector<double> u, f(5, 0.0);
    const svxg_pcg_result r = P.solve(f, u, 1e-9, 100, false);
    CHECK(r.breakdown && !r.converged && std::isinf(r.rel_res));
    CHECK(!P.error().empty());
    svxg::StressProblem Q;
    cantilever(Q, 4, 0.5, 100.0);
    Q.mats.resize(3);  // (an incomplete material table: assemble refuses, nothing throws)
    CHECK(!Q.assemble());
  }
  std::printf(failures ? "%d failures\n" : "ok\n", failures);
  return failures ? 1 : 0;
}
