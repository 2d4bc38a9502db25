// test_svx_binding.cpp - the reference-side binding (include/svxg_svx.hpp) compiled against the
// reference's own headers and linked with the reference's compiled stress sources (the oracle's
// libsvxref.so) and this library (libsvxg.so).
//
// Host part (every run): the records convert field by field; the library's bond_utilization and
// add_force give the reference's numbers bit for bit on the reference's own types; the pinned
// node is the nearest one. Device part (when a GPU is present): World::Impl::probe_utilization
// (core/src/world/world.cpp:1907-1940) run on svx::StressProblem and on svx::GpuStressProblem -
// load_vector, assemble, solve to 1e-8 warm, bond_utilization of every intact bond through
// bond_load bond by bond - the same worst utilization (1e-6) and the same count over strength,
// in one device pass of bond loads; then one bond removed on both and the probe again.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "svxg_svx.hpp"

using namespace svx;

namespace {

int failures = 0;
#define CHECK(c)                                                 \
  do {                                                           \
    if (!(c)) {                                                  \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                \
    }                                                            \
  } while (0)

// a bond as the reference's tests make one (tests/core/test_stress.cpp:14-32): a square section
// of side a at p, normal n
SBond make_bond(const std::vector<SNode>& nodes, i32 A, i32 B, V3 n, V3 p, f64 a, MaterialId m) {
  SBond s;
  s.a = A;
  s.b = B;
  s.ma = s.mb = m;
  s.n = n;
  s.t1 = std::fabs(n.x) > 0.5 ? V3{0, 1, 0} : V3{1, 0, 0};
  s.t2 = cross(n, s.t1);
  s.area = a * a;
  s.p = p;
  s.s1 = s.s2 = a * a * a * a / 12.0;
  s.c1 = s.c2 = 0.5 * a;
  s.rmax = std::sqrt(0.5) * a;
  s.la = std::fabs(dot(p - nodes[size_t(A)].c, n));
  s.lb = B >= 0 ? std::fabs(dot(nodes[size_t(B)].c - p, n)) : s.la;
  s.faces = 16;
  return s;
}

// a tower of nx x ny x nz cells (0.5 m) on supports under z = 0, with a few sectioned bonds
template <class P>
void tower(P& G, int nx, int ny, int nz) {
  const f64 h = 0.5;
  auto id = [&](int x, int y, int z) { return i32((z * ny + y) * nx + x); };
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        SNode nd;
        nd.c = V3{(x + 0.5) * h, (y + 0.5) * h, (z + 0.5) * h};
        nd.mass = 300.0 + 10.0 * ((x + 2 * y + 3 * z) % 7);
        G.nodes.push_back(nd);
      }
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const V3 c = G.nodes[size_t(id(x, y, z))].c;
        const MaterialId m = ((x + y + z) % 3) == 0 ? MaterialId::Rc : MaterialId::Concrete;
        if (z == 0) G.bonds.push_back(make_bond(G.nodes, id(x, y, z), -1, {0, 0, -1}, {c.x, c.y, 0.0}, h, m));
        if (x + 1 < nx) G.bonds.push_back(make_bond(G.nodes, id(x, y, z), id(x + 1, y, z), {1, 0, 0}, {c.x + 0.5 * h, c.y, c.z}, h, m));
        if (y + 1 < ny) G.bonds.push_back(make_bond(G.nodes, id(x, y, z), id(x, y + 1, z), {0, 1, 0}, {c.x, c.y + 0.5 * h, c.z}, h, m));
        if (z + 1 < nz) G.bonds.push_back(make_bond(G.nodes, id(x, y, z), id(x, y, z + 1), {0, 0, 1}, {c.x, c.y, c.z + 0.5 * h}, h, m));
      }
  for (size_t k = 0; k < G.bonds.size(); k += 5) {
    SBond& b = G.bonds[k];
    b.sectioned = true;
    b.ft = 0.9e6f;
    b.fb = 1.5e6f;
    b.fc = 2.0e7f;
    b.coh = 1.1e6f;
    b.mu = 0.6f;
    b.strength = 0.8 + 0.05 * f64(k % 9);
  }
}

std::vector<f64> weights(const std::vector<SNode>& nodes) {
  std::vector<f64> w(nodes.size());
  for (size_t i = 0; i < nodes.size(); ++i) w[i] = nodes[i].fixed ? 0.0 : nodes[i].mass * 9.81;
  return w;
}

// World::Impl::probe_utilization's loop (world.cpp:1920-1933) on either problem type
template <class P>
f64 probe(P& G, std::vector<f64>& u, f64 fragility, i32* over, const StressOptions& so) {
  const std::vector<f64> F = gpu_load_vector(weights(G.nodes), std::vector<f64>(6 * G.nodes.size(), 0.0));
  if (!G.assembled()) G.assemble(so);
  G.solve(F, u, 1e-8, 5000, true);
  f64 mx = 0.0;
  i32 cnt = 0;
  for (i32 b = 0; b < static_cast<i32>(G.bonds.size()); ++b) {
    if (G.bonds[size_t(b)].broken) continue;
    const f64 phi = bond_utilization(G.bonds[size_t(b)], G.bond_load(b, u), fragility, G.materials());
    mx = std::max(mx, phi);
    cnt += phi >= 1.0 ? 1 : 0;
  }
  *over = cnt;
  return mx;
}

}  // namespace

int main() {
  const MaterialTable& table = default_materials();
  const std::vector<svxg_material> mats = to_svxg(table);
  StressProblem R;
  tower(R, 4, 4, 12);

  // records: field by field, the reference's order kept where it differs
  {
    const SBond& s = R.bonds[5];
    const svxg_bond b = to_svxg(s);
    CHECK(b.a == s.a && b.b == s.b && b.ma == u8(s.ma) && b.sectioned == 1 && b.ft == s.ft && b.mu == s.mu);
    CHECK(b.area == s.area && b.s1 == s.s1 && b.la == s.la && b.strength == s.strength && b.tag == s.tag);
    const svxg_node n = to_svxg(R.nodes[7]);
    CHECK(n.c.x == R.nodes[7].c.x && n.mass == R.nodes[7].mass && n.fixed == 0);
    CHECK(mats.size() == SVXG_MAX_MATERIALS && mats[1].ft == table[MaterialId::Concrete].ft);
    CHECK(mats[SVXG_MAX_MATERIALS - 1].E == table[static_cast<MaterialId>(0)].E);  // (unregistered: id 0's)
  }
  // bond_utilization (stress.cpp:23-57): the library's host function against the reference's,
  // every bond under random loads at random fragilities, bit for bit
  {
    std::mt19937_64 rng(17);
    std::uniform_real_distribution<f64> mag(1.0, 6.0), sgn(-1.0, 1.0), frag(0.3, 3.0);
    int modes[4] = {0, 0, 0, 0};
    for (int rep = 0; rep < 8; ++rep)
      for (const SBond& s : R.bonds) {
        BondLoad L;
        f64* v[6] = {&L.N, &L.V1, &L.V2, &L.T, &L.M1, &L.M2};
        for (f64* x : v) *x = sgn(rng) * std::pow(10.0, mag(rng));
        const f64 fr = frag(rng);
        FailMode m = FailMode::None;
        uint8_t gm = 9;
        const f64 a = bond_utilization(s, L, fr, table, &m);
        const svxg_bond gb = to_svxg(s);
        const svxg_bond_load gl = to_svxg(L);
        const f64 b = svxg_bond_utilization(&gb, &gl, fr, mats.data(), &gm);
        CHECK(a == b && u8(m) == gm);
        ++modes[gm & 3];
      }
    CHECK(modes[1] > 0 && modes[2] > 0 && modes[3] > 0);
  }
  // add_force (stress.cpp:504-513): the same bits as the reference's
  {
    std::vector<f64> fa(6 * R.nodes.size(), 0.0), fb = fa;
    for (i32 i = 0; i < 40; ++i) {
      const V3 F{1e3 * i - 7.5, 3.25 * i, -1e4 + i}, at{0.1 * i, 2.0 - 0.3 * i, 1.7};
      StressProblem::add_force(fa, i % 30, R.nodes[size_t(i % 30)].c, F, at);
      GpuStressProblem::add_force(fb, i % 30, R.nodes[size_t(i % 30)].c, F, at);
    }
    CHECK(fa == fb);
  }
  // pin_reference (world_pieces.cpp:313-326): the node nearest the centre of mass, the only one fixed
  {
    std::vector<SNode> n = R.nodes;
    n[3].fixed = true;
    const V3 com{1.1, 0.9, 2.6};
    const i32 pin = gpu_pin_reference(n, com);
    i32 want = 0;
    for (i32 i = 1; i < i32(n.size()); ++i)
      if (norm2(n[size_t(i)].c - com) < norm2(n[size_t(want)].c - com)) want = i;
    CHECK(pin == want && n[size_t(pin)].fixed && !n[3].fixed);
  }

  GpuStressProblem G;
  if (!G.ok()) {
    std::printf("device part skipped (%s)\n", G.error().c_str());
  } else {
    tower(G, 4, 4, 12);
    StressOptions so;
    so.rtol = 1e-3;
    so.amg_min_nodes = 32;  // (a multigrid on both sides)
    const f64 fragility = 0.02;  // (this tower is far from its strength: a tenth or so over it)
    std::vector<f64> ur, ug;
    i32 over_r = 0, over_g = 0;
    const f64 mr = probe(R, ur, fragility, &over_r, so);
    const f64 mg = probe(G, ug, fragility, &over_g, so);
    std::printf("probe: reference max phi %.9g over %d, device %.9g over %d, %lld bond-load pass(es)\n", mr, over_r, mg,
                over_g, (long long)G.device().bond_load_passes());
    CHECK(std::fabs(mr - mg) <= 1e-6 * mr && over_r == over_g && over_r > 0);
    CHECK(G.device().bond_load_passes() == 1);
    // a bond removed in place (stress.hpp:105): the flags come back, the probe agrees again
    R.remove_bond(7);
    G.remove_bond(7);
    CHECK(G.bonds[7].broken && !G.bonds[7].in_k && R.bonds[7].broken);
    const f64 mr2 = probe(R, ur, fragility, &over_r, so);
    const f64 mg2 = probe(G, ug, fragility, &over_g, so);
    CHECK(std::fabs(mr2 - mg2) <= 1e-6 * mr2 && over_r == over_g);
    CHECK(G.memory_bytes() > G.solver_bytes() && G.solver_bytes() > 0);
  }
  std::printf(failures ? "%d failures\n" : "ok\n", failures);
  return failures ? 1 : 0;
}
