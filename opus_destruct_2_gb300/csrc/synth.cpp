// synth.cpp - seeded synthetic fragment graphs for the stress solve's workloads (host code).
//
// The reference builds its graphs from voxels (its fragmenter core/src/frag/fragments.cpp and
// the section geometry of core/src/world/world_internal.hpp:133-360); neither is on the solve
// path. This generator makes graphs of the same kind directly:
//   1. an occupancy grid of h = 0.5 m voxels (storey frames: slabs, perimeter walls with
//      openings, columns, a walled core; or a random connected blob for a loose piece);
//   2. fragments: the connected parts of the occupied voxels inside jittered cells 2-3 voxels a
//      side (about 4-27 voxels each), parts under 4 voxels merged into the neighbour they share
//      most faces with;
//   3. bonds: one per face-adjacent pair of fragments, along the axis of most shared faces, with
//      area = faces x h^2, p = the faces' centroid, a square section of side sqrt(area)
//      (s1 = s2 = a^4 / 12, c1 = c2 = a / 2, rmax = a / sqrt 2), the local frame of the
//      reference's own test fixture (tests/core/test_stress.cpp:14-32), la / lb from the
//      fragments' centres; supports (b = -1) on the ground faces;
//   4. loads: gravity on every fragment (mass = density x volume) plus, for pieces, one seeded
//      impact force; a free piece carries inertial-relief loads (its rigid acceleration taken
//      out, as core/src/world/world_pieces.cpp:566-597) and its node nearest the centre of mass
//      is pinned (world_pieces.cpp:313-326).
// Randomness: std::mt19937_64 with the seed, mapped to doubles by its top 53 bits.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "svxg_types.h"

namespace {

constexpr double kVoxel = 0.5;

struct Rng {
  std::mt19937_64 g;
  explicit Rng(uint64_t s) : g(s) {}
  double uniform() { return static_cast<double>(g() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  int64_t integer(int64_t lo, int64_t hi) { return lo + static_cast<int64_t>(uniform() * double(hi - lo + 1)); }
  double normal() {
    const double u1 = std::max(uniform(), 1e-300), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

// A voxel structure: a dense occupancy box with a material id and strength jitter base.
struct Grid {
  int nx = 0, ny = 0, nz = 0;
  double ox = 0, oy = 0;          // world offset of voxel (0, 0, 0) (m)
  std::vector<uint8_t> occ;       // 1: occupied
  uint8_t mat = 0;
  bool grounded = true;           // voxels at z = 0 stand on supports
  size_t at(int x, int y, int z) const { return (size_t(z) * ny + y) * nx + x; }
  bool on(int x, int y, int z) const {
    return x >= 0 && y >= 0 && z >= 0 && x < nx && y < ny && z < nz && occ[at(x, y, z)];
  }
};

struct Graph {
  std::vector<svxg_node> nodes;
  std::vector<svxg_bond> bonds;
  std::vector<double> f;
  // the same bonds as interfaces of voxel faces (the section-geometry path)
  std::vector<svxg_section> secs;
  std::vector<svxg_face> faces;
};

// Tower frame: storeys of `hs` voxels, slabs `ts` thick, a perimeter wall two voxels thick with
// openings, interior cross walls with doors, 2 x 2 columns every `span` voxels, a walled core.
Grid tower_grid(int wx, int wy, int storeys, Rng& R) {
  Grid G;
  const int hs = 8, ts = 2, span = 6;
  G.nx = wx;
  G.ny = wy;
  G.nz = storeys * hs + ts;
  G.occ.assign(size_t(G.nx) * G.ny * G.nz, 0);
  auto set = [&](int x, int y, int z) {
    if (x >= 0 && y >= 0 && z >= 0 && x < G.nx && y < G.ny && z < G.nz) G.occ[G.at(x, y, z)] = 1;
  };
  for (int s = 0; s <= storeys; ++s) {
    const int z0 = s * hs;
    for (int z = z0; z < z0 + ts; ++z)
      for (int y = 0; y < wy; ++y)
        for (int x = 0; x < wx; ++x) set(x, y, z);
    if (s == storeys) break;
    // walls with window openings (2 wide, 2 high, random)
    for (int z = z0 + ts; z < z0 + hs; ++z) {
      for (int x = 0; x < wx; ++x) {
        set(x, 0, z);
        set(x, 1, z);
        set(x, wy - 2, z);
        set(x, wy - 1, z);
      }
      for (int y = 0; y < wy; ++y) {
        set(0, y, z);
        set(1, y, z);
        set(wx - 2, y, z);
        set(wx - 1, y, z);
      }
    }
    const int nwin = (wx + wy) / 4;
    for (int w = 0; w < nwin; ++w) {
      const int side = int(R.integer(0, 3));
      const int len = side < 2 ? wx : wy;
      if (len < 6) continue;
      const int p0 = int(R.integer(2, len - 4));
      for (int z = z0 + ts + 2; z < z0 + ts + 4 && z < z0 + hs; ++z)
        for (int p = p0; p < p0 + 2; ++p) {
          int x = 0, y = 0;
          for (int t = 0; t < 2; ++t) {
            if (side == 0) { x = p; y = t; }
            else if (side == 1) { x = p; y = wy - 1 - t; }
            else if (side == 2) { x = t; y = p; }
            else { x = wx - 1 - t; y = p; }
            G.occ[G.at(x, y, z)] = 0;
          }
        }
    }
    // interior cross walls (two voxels thick) with a door in each half
    for (int z = z0 + ts; z < z0 + hs; ++z) {
      const bool door = z < z0 + ts + 5;
      for (int x = 2; x < wx - 2; ++x)
        if (!(door && (x == wx / 4 || x == wx / 4 + 1 || x == 3 * wx / 4 || x == 3 * wx / 4 + 1))) {
          set(x, wy / 2 - 1, z);
          set(x, wy / 2, z);
        }
      for (int y = 2; y < wy - 2; ++y)
        if (!(door && (y == wy / 4 || y == wy / 4 + 1 || y == 3 * wy / 4 || y == 3 * wy / 4 + 1))) {
          set(wx / 2 - 1, y, z);
          set(wx / 2, y, z);
        }
    }
    // columns
    for (int cx = span; cx < wx - 1; cx += span)
      for (int cy = span; cy < wy - 1; cy += span)
        for (int z = z0 + ts; z < z0 + hs; ++z)
          for (int t = 0; t < 4; ++t) set(cx + t % 2, cy + t / 2, z);
    // core: a 4 x 4 shaft in the middle, one door
    const int kx = wx / 2 - 2, ky = wy / 2 - 2;
    if (wx >= 12 && wy >= 12)
      for (int z = z0 + ts; z < z0 + hs; ++z)
        for (int i = 0; i < 4; ++i) {
          set(kx + i, ky, z);
          set(kx + i, ky + 3, z);
          set(kx, ky + i, z);
          if (!(i == 1 || i == 2) || z >= z0 + ts + 4) set(kx + 3, ky + i, z);
        }
  }
  return G;
}

// A random connected blob of about `voxels` voxels (Eden growth, biased to elongated shapes).
Grid blob_grid(int64_t voxels, Rng& R) {
  const int side = int(std::ceil(std::cbrt(double(voxels)) * 2.2)) + 4;
  Grid G;
  G.nx = G.ny = G.nz = side;
  G.occ.assign(size_t(side) * side * side, 0);
  std::vector<std::array<int, 3>> front;
  const int c = side / 2;
  G.occ[G.at(c, c, c)] = 1;
  front.push_back({c, c, c});
  int64_t count = 1;
  const double stretch[3] = {R.uniform(0.5, 1.5), R.uniform(0.5, 1.5), R.uniform(0.5, 1.5)};
  static const int dirs[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  while (count < voxels && !front.empty()) {
    const size_t k = size_t(R.integer(0, int64_t(front.size()) - 1));
    const auto v = front[k];
    double wsum = 0;
    for (int d = 0; d < 6; ++d) wsum += stretch[d / 2];
    double pick = R.uniform() * wsum;
    int d = 0;
    for (; d < 5; ++d) {
      pick -= stretch[d / 2];
      if (pick < 0) break;
    }
    const int x = v[0] + dirs[d][0], y = v[1] + dirs[d][1], z = v[2] + dirs[d][2];
    if (x < 1 || y < 1 || z < 1 || x >= side - 1 || y >= side - 1 || z >= side - 1) {
      front[k] = front.back();
      front.pop_back();
      continue;
    }
    if (!G.occ[G.at(x, y, z)]) {
      G.occ[G.at(x, y, z)] = 1;
      front.push_back({x, y, z});
      ++count;
    }
  }
  // drop it to the floor: lowest occupied z becomes 0
  int zmin = side;
  for (int z = 0; z < side && zmin == side; ++z)
    for (int y = 0; y < side && zmin == side; ++y)
      for (int x = 0; x < side; ++x)
        if (G.occ[G.at(x, y, z)]) {
          zmin = z;
          break;
        }
  if (zmin > 0 && zmin < side) {
    std::vector<uint8_t> o(G.occ.size(), 0);
    for (int z = zmin; z < side; ++z)
      for (int y = 0; y < side; ++y)
        for (int x = 0; x < side; ++x) o[G.at(x, y, z - zmin)] = G.occ[G.at(x, y, z)];
    G.occ.swap(o);
  }
  return G;
}

struct MatProps {
  double rho, ft, fb, fc, coh, mu;
};

// Fragments, bonds and gravity loads of a grid, appended to g.
void fragment(const Grid& G, const MatProps& M, Rng& R, Graph& g) {
  const size_t nvox = G.occ.size();
  // jittered cell boundaries along each axis: steps of 2-3 voxels
  auto cuts = [&](int n) {
    std::vector<int> cell(static_cast<size_t>(n));
    int c = 0, left = int(R.integer(2, 3));
    for (int i = 0; i < n; ++i) {
      cell[size_t(i)] = c;
      if (--left == 0) {
        ++c;
        left = int(R.integer(2, 3));
      }
    }
    return cell;
  };
  const std::vector<int> cx = cuts(G.nx), cy = cuts(G.ny), cz = cuts(G.nz);
  std::vector<int32_t> frag(nvox, -1);
  std::vector<int32_t> size;
  std::vector<size_t> stack;
  // connected parts within a cell, in cell order (z, y, x of the cells) for locality
  const int ncx = cx.back() + 1, ncy = cy.back() + 1, ncz = cz.back() + 1;
  std::vector<std::vector<size_t>> bycell(size_t(ncx) * ncy * ncz);
  for (int z = 0; z < G.nz; ++z)
    for (int y = 0; y < G.ny; ++y)
      for (int x = 0; x < G.nx; ++x)
        if (G.occ[G.at(x, y, z)])
          bycell[(size_t(cz[size_t(z)]) * ncy + cy[size_t(y)]) * ncx + cx[size_t(x)]].push_back(G.at(x, y, z));
  static const int dirs[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  auto coords = [&](size_t v, int& x, int& y, int& z) {
    x = int(v % size_t(G.nx));
    y = int((v / size_t(G.nx)) % size_t(G.ny));
    z = int(v / (size_t(G.nx) * G.ny));
  };
  for (const auto& cell : bycell)
    for (size_t v0 : cell) {
      if (frag[v0] >= 0) continue;
      const int32_t id = int32_t(size.size());
      size.push_back(0);
      frag[v0] = id;
      stack.push_back(v0);
      int x0, y0, z0;
      coords(v0, x0, y0, z0);
      const int kx = cx[size_t(x0)], ky = cy[size_t(y0)], kz = cz[size_t(z0)];
      while (!stack.empty()) {
        const size_t v = stack.back();
        stack.pop_back();
        ++size[size_t(id)];
        int x, y, z;
        coords(v, x, y, z);
        for (const auto& d : dirs) {
          const int a = x + d[0], b = y + d[1], c = z + d[2];
          if (!G.on(a, b, c)) continue;
          if (cx[size_t(a)] != kx || cy[size_t(b)] != ky || cz[size_t(c)] != kz) continue;
          const size_t w = G.at(a, b, c);
          if (frag[w] < 0) {
            frag[w] = id;
            stack.push_back(w);
          }
        }
      }
    }
  // merge parts under 4 voxels into the face-neighbour they share most faces with
  const int32_t nf0 = int32_t(size.size());
  std::vector<int32_t> remap(static_cast<size_t>(nf0));
  for (int32_t i = 0; i < nf0; ++i) remap[size_t(i)] = i;
  auto root = [&](int32_t i) {
    while (remap[size_t(i)] != i) i = remap[size_t(i)];
    return i;
  };
  {
    std::vector<std::map<int32_t, int>> shared(static_cast<size_t>(nf0));
    for (int z = 0; z < G.nz; ++z)
      for (int y = 0; y < G.ny; ++y)
        for (int x = 0; x < G.nx; ++x) {
          if (!G.occ[G.at(x, y, z)]) continue;
          const int32_t a = frag[G.at(x, y, z)];
          if (size[size_t(a)] >= 4) continue;
          for (const auto& d : dirs) {
            const int p = x + d[0], q = y + d[1], r = z + d[2];
            if (!G.on(p, q, r)) continue;
            const int32_t b = frag[G.at(p, q, r)];
            if (b != a) ++shared[size_t(a)][b];
          }
        }
    for (int32_t a = 0; a < nf0; ++a) {
      if (size[size_t(a)] >= 4 || shared[size_t(a)].empty()) continue;
      int32_t best = -1;
      int bc = -1;
      for (const auto& e : shared[size_t(a)])
        if (e.second > bc) {
          bc = e.second;
          best = e.first;
        }
      const int32_t rb = root(best);
      if (rb != a) remap[size_t(a)] = rb;
    }
  }
  // final numbering in first-appearance order of the roots
  std::vector<int32_t> idmap(size_t(nf0), -1);
  const int32_t base = int32_t(g.nodes.size());
  int32_t nf = 0;
  for (int32_t i = 0; i < nf0; ++i) {
    const int32_t r = root(i);
    if (idmap[size_t(r)] < 0) idmap[size_t(r)] = nf++;
  }
  for (size_t v = 0; v < nvox; ++v)
    if (frag[v] >= 0) frag[v] = idmap[size_t(root(frag[v]))];
  // node centres and masses
  std::vector<double> sx(size_t(nf), 0), sy(size_t(nf), 0), sz(size_t(nf), 0);
  std::vector<int64_t> cnt(size_t(nf), 0);
  for (int z = 0; z < G.nz; ++z)
    for (int y = 0; y < G.ny; ++y)
      for (int x = 0; x < G.nx; ++x) {
        const int32_t a = frag[G.at(x, y, z)];
        if (a < 0) continue;
        sx[size_t(a)] += G.ox + (x + 0.5) * kVoxel;
        sy[size_t(a)] += G.oy + (y + 0.5) * kVoxel;
        sz[size_t(a)] += (z + 0.5) * kVoxel;
        ++cnt[size_t(a)];
      }
  const double vvol = kVoxel * kVoxel * kVoxel;
  for (int32_t a = 0; a < nf; ++a) {
    svxg_node nd;
    std::memset(&nd, 0, sizeof(nd));
    nd.c = {sx[size_t(a)] / double(cnt[size_t(a)]), sy[size_t(a)] / double(cnt[size_t(a)]),
            sz[size_t(a)] / double(cnt[size_t(a)])};
    nd.mass = M.rho * double(cnt[size_t(a)]) * vvol;
    g.nodes.push_back(nd);
    double* fi = nullptr;
    g.f.resize(g.f.size() + 6, 0.0);
    fi = &g.f[g.f.size() - 6];
    fi[2] = -9.81 * nd.mass;
  }
  // shared faces per pair and axis: count, centroid sum, orientation sum
  struct Faces {
    int n[3] = {0, 0, 0};
    double px[3] = {0, 0, 0}, py[3] = {0, 0, 0}, pz[3] = {0, 0, 0};
    int sgn[3] = {0, 0, 0};
  };
  std::map<std::pair<int32_t, int32_t>, Faces> pairs;
  std::vector<int> ground(size_t(nf), 0);
  std::vector<double> gx(size_t(nf), 0), gy(size_t(nf), 0);
  for (int z = 0; z < G.nz; ++z)
    for (int y = 0; y < G.ny; ++y)
      for (int x = 0; x < G.nx; ++x) {
        const int32_t a = frag[G.at(x, y, z)];
        if (a < 0) continue;
        if (z == 0 && G.grounded) {
          ++ground[size_t(a)];
          gx[size_t(a)] += G.ox + (x + 0.5) * kVoxel;
          gy[size_t(a)] += G.oy + (y + 0.5) * kVoxel;
        }
        for (int ax = 0; ax < 3; ++ax) {
          const int p = x + (ax == 0), q = y + (ax == 1), r = z + (ax == 2);
          if (!G.on(p, q, r)) continue;
          const int32_t b = frag[G.at(p, q, r)];
          if (b == a) continue;
          const bool fwd = a < b;
          Faces& F = pairs[fwd ? std::make_pair(a, b) : std::make_pair(b, a)];
          ++F.n[ax];
          F.sgn[ax] += fwd ? 1 : -1;
          F.px[ax] += G.ox + (x + 0.5 + 0.5 * (ax == 0)) * kVoxel;
          F.py[ax] += G.oy + (y + 0.5 + 0.5 * (ax == 1)) * kVoxel;
          F.pz[ax] += (z + 0.5 + 0.5 * (ax == 2)) * kVoxel;
        }
      }
  auto section = [&](svxg_bond& s, double area) {
    const double a = std::sqrt(area);
    s.area = area;
    s.s1 = s.s2 = a * a * a * a / 12.0;
    s.c1 = s.c2 = 0.5 * a;
    s.rmax = std::sqrt(0.5) * a;
    s.strength = 1.0;
    s.sectioned = 1;
    s.ft = float(M.ft * R.uniform(0.9, 1.1));
    s.fb = float(M.fb * R.uniform(0.9, 1.1));
    s.fc = float(M.fc * R.uniform(0.9, 1.1));
    s.coh = float(M.coh * R.uniform(0.9, 1.1));
    s.mu = float(M.mu);
    s.ma = s.mb = G.mat;
    s.tag = -1;
  };
  auto frame = [](svxg_bond& s, const double n[3]) {
    s.n = {n[0], n[1], n[2]};
    const double t1[3] = {std::abs(n[0]) > 0.5 ? 0.0 : 1.0, std::abs(n[0]) > 0.5 ? 1.0 : 0.0, 0.0};
    s.t1 = {t1[0], t1[1], t1[2]};
    s.t2 = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
  };
  auto dotp = [](const svxg_v3& a, const double n[3]) { return a.x * n[0] + a.y * n[1] + a.z * n[2]; };
  // supports first for each fragment in order, then the pairs in (a, b) order
  std::vector<std::vector<svxg_bond>> per(static_cast<size_t>(nf));
  for (int32_t a = 0; a < nf; ++a) {
    if (!ground[size_t(a)]) continue;
    svxg_bond s;
    std::memset(&s, 0, sizeof(s));
    s.a = base + a;
    s.b = -1;
    const double n[3] = {0, 0, -1};
    frame(s, n);
    s.p = {gx[size_t(a)] / ground[size_t(a)], gy[size_t(a)] / ground[size_t(a)], 0.0};
    section(s, ground[size_t(a)] * kVoxel * kVoxel);
    const svxg_node& na = g.nodes[size_t(base + a)];
    const svxg_v3 d = {s.p.x - na.c.x, s.p.y - na.c.y, s.p.z - na.c.z};
    s.la = std::abs(dotp(d, n));
    s.lb = s.la;
    s.faces = ground[size_t(a)];
    per[size_t(a)].push_back(s);
  }
  for (const auto& e : pairs) {
    const Faces& F = e.second;
    int ax = 0;
    for (int k = 1; k < 3; ++k)
      if (F.n[k] > F.n[ax]) ax = k;
    svxg_bond s;
    std::memset(&s, 0, sizeof(s));
    s.a = base + e.first.first;
    s.b = base + e.first.second;
    double n[3] = {0, 0, 0};
    n[ax] = F.sgn[ax] >= 0 ? 1.0 : -1.0;
    frame(s, n);
    s.p = {F.px[ax] / F.n[ax], F.py[ax] / F.n[ax], F.pz[ax] / F.n[ax]};
    section(s, F.n[ax] * kVoxel * kVoxel);
    const svxg_node& na = g.nodes[size_t(s.a)];
    const svxg_node& nb = g.nodes[size_t(s.b)];
    const svxg_v3 da = {s.p.x - na.c.x, s.p.y - na.c.y, s.p.z - na.c.z};
    const svxg_v3 db = {nb.c.x - s.p.x, nb.c.y - s.p.y, nb.c.z - s.p.z};
    s.la = std::abs(dotp(da, n));
    s.lb = std::abs(dotp(db, n));
    s.faces = F.n[ax];
    per[size_t(e.first.first)].push_back(s);
  }
  for (auto& v : per)
    for (auto& s : v) g.bonds.push_back(s);
  // The interfaces of the same bonds (in the same order) as the world accumulates them: every
  // face two fragments share, of any axis, in scan order; a grounded fragment's faces on the
  // ground below it. Voxel damage: one voxel in eight, 1-200, from its own seeded stream (the
  // graph's stream is left as it was).
  const int ix0 = int(std::lround(G.ox / kVoxel)), iy0 = int(std::lround(G.oy / kVoxel));
  Rng D(0x5EC7u ^ (uint64_t(uint32_t(base)) << 20) ^ (uint64_t(G.nx) << 8) ^ uint64_t(G.nz));
  std::vector<uint8_t> dmg(nvox, 0);
  for (size_t v = 0; v < nvox; ++v)
    if (G.occ[v] && D.integer(0, 7) == 0) dmg[v] = uint8_t(D.integer(1, 200));
  const uint8_t vox = uint8_t(G.mat + 1);
  const uint8_t rock_vox = uint8_t((5 + 1) | 0x80);  // (rock, anchored)
  std::vector<std::vector<svxg_face>> sup(static_cast<size_t>(nf));
  std::map<std::pair<int32_t, int32_t>, std::vector<svxg_face>> acc;
  for (int z = 0; z < G.nz; ++z)
    for (int y = 0; y < G.ny; ++y)
      for (int x = 0; x < G.nx; ++x) {
        const size_t v = G.at(x, y, z);
        const int32_t a = frag[v];
        if (a < 0) continue;
        if (z == 0 && G.grounded) {
          svxg_face fc;
          std::memset(&fc, 0, sizeof(fc));
          fc.x = x + ix0;
          fc.y = y + iy0;
          fc.z = -1;
          fc.axis = 2;
          fc.sign = -1;
          fc.vox_lo = rock_vox;
          fc.vox_hi = vox;
          fc.damage_hi = dmg[v];
          sup[size_t(a)].push_back(fc);
        }
        for (int ax = 0; ax < 3; ++ax) {
          const int p = x + (ax == 0), q = y + (ax == 1), r = z + (ax == 2);
          if (!G.on(p, q, r)) continue;
          const size_t w = G.at(p, q, r);
          const int32_t b = frag[w];
          if (b == a) continue;
          svxg_face fc;
          std::memset(&fc, 0, sizeof(fc));
          fc.x = x + ix0;
          fc.y = y + iy0;
          fc.z = z;
          fc.axis = uint8_t(ax);
          fc.sign = a < b ? 1 : -1;
          fc.vox_lo = vox;
          fc.vox_hi = vox;
          fc.damage_lo = dmg[v];
          fc.damage_hi = dmg[w];
          acc[a < b ? std::make_pair(a, b) : std::make_pair(b, a)].push_back(fc);
        }
      }
  auto emit = [&](int32_t a, int32_t b, const std::vector<svxg_face>& fs) {
    svxg_section sc;
    std::memset(&sc, 0, sizeof(sc));
    sc.a = base + a;
    sc.b = b >= 0 ? base + b : -1;
    sc.first_face = int64_t(g.faces.size());
    sc.faces = int32_t(fs.size());
    sc.axis = 2;
    sc.sign = -1;
    sc.ma = G.mat;
    sc.mb = b >= 0 ? G.mat : uint8_t(5);
    sc.sectioned = 1;
    sc.h = kVoxel;
    sc.strength_a = 1.0;
    sc.strength_b = b >= 0 ? 1.0 : 1e9;  // (the anchored side never governs)
    g.secs.push_back(sc);
    g.faces.insert(g.faces.end(), fs.begin(), fs.end());
  };
  {
    auto it = acc.begin();
    for (int32_t a = 0; a < nf; ++a) {
      if (!sup[size_t(a)].empty()) emit(a, -1, sup[size_t(a)]);
      for (; it != acc.end() && it->first.first == a; ++it) emit(a, it->first.second, it->second);
    }
  }
}

// Loads of a free piece: its rigid acceleration under gravity and the impact taken out of every
// fragment's load, the node nearest the centre of mass pinned.
void free_body(Graph& g, size_t n0, int32_t impact_node, const double F[3]) {
  const size_t n1 = g.nodes.size();
  double M = 0, cx = 0, cy = 0, cz = 0;
  for (size_t i = n0; i < n1; ++i) {
    M += g.nodes[i].mass;
    cx += g.nodes[i].mass * g.nodes[i].c.x;
    cy += g.nodes[i].mass * g.nodes[i].c.y;
    cz += g.nodes[i].mass * g.nodes[i].c.z;
  }
  cx /= M;
  cy /= M;
  cz /= M;
  // inertia of point masses about the centre, torque of the impact
  double I[9] = {0};
  for (size_t i = n0; i < n1; ++i) {
    const double r[3] = {g.nodes[i].c.x - cx, g.nodes[i].c.y - cy, g.nodes[i].c.z - cz};
    const double m = g.nodes[i].mass, rr = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) I[3 * a + b] += m * ((a == b ? rr : 0.0) - r[a] * r[b]);
  }
  for (int a = 0; a < 3; ++a) I[4 * a] += 1e-9 * M;
  double tau[3] = {0, 0, 0};
  if (impact_node >= 0) {
    const svxg_node& p = g.nodes[size_t(impact_node)];
    const double r[3] = {p.c.x - cx, p.c.y - cy, p.c.z - cz};
    tau[0] = r[1] * F[2] - r[2] * F[1];
    tau[1] = r[2] * F[0] - r[0] * F[2];
    tau[2] = r[0] * F[1] - r[1] * F[0];
  }
  // alpha = I^-1 tau (Cramer)
  const double det = I[0] * (I[4] * I[8] - I[5] * I[7]) - I[1] * (I[3] * I[8] - I[5] * I[6]) +
                     I[2] * (I[3] * I[7] - I[4] * I[6]);
  double al[3] = {0, 0, 0};
  if (std::abs(det) > 0) {
    const double inv[9] = {(I[4] * I[8] - I[5] * I[7]) / det, (I[2] * I[7] - I[1] * I[8]) / det,
                           (I[1] * I[5] - I[2] * I[4]) / det, (I[5] * I[6] - I[3] * I[8]) / det,
                           (I[0] * I[8] - I[2] * I[6]) / det, (I[2] * I[3] - I[0] * I[5]) / det,
                           (I[3] * I[7] - I[4] * I[6]) / det, (I[1] * I[6] - I[0] * I[7]) / det,
                           (I[0] * I[4] - I[1] * I[3]) / det};
    for (int a = 0; a < 3; ++a) al[a] = inv[3 * a] * tau[0] + inv[3 * a + 1] * tau[1] + inv[3 * a + 2] * tau[2];
  }
  const double acc[3] = {F[0] / M, F[1] / M, F[2] / M - 9.81};
  size_t pin = n0;
  double best = 1e300;
  for (size_t i = n0; i < n1; ++i) {
    const double r[3] = {g.nodes[i].c.x - cx, g.nodes[i].c.y - cy, g.nodes[i].c.z - cz};
    const double m = g.nodes[i].mass;
    const double axr[3] = {al[1] * r[2] - al[2] * r[1], al[2] * r[0] - al[0] * r[2], al[0] * r[1] - al[1] * r[0]};
    double* fi = &g.f[6 * i];
    fi[0] = m * (0.0 - acc[0] - axr[0]);
    fi[1] = m * (0.0 - acc[1] - axr[1]);
    fi[2] = m * (-9.81 - acc[2] - axr[2]);
    const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    if (d2 < best) {
      best = d2;
      pin = i;
    }
  }
  if (impact_node >= 0)
    for (int a = 0; a < 3; ++a) g.f[6 * size_t(impact_node) + a] += F[a];
  g.nodes[pin].fixed = 1;
}

struct Handle {
  Graph g;
};

}  // namespace

extern "C" {

// Material of a tower: solve-side density and strengths (the caller's material table holds E/G).
typedef struct svxs_material {
  double rho, ft, fb, fc, coh, mu;
  int32_t id;
  int32_t pad;
} svxs_material;

// One tower of `storeys` storeys, `wx` x `wy` voxels in plan at (ox, oy) m.
void* svxs_tower(int32_t wx, int32_t wy, int32_t storeys, double ox, double oy, const svxs_material* m,
                 uint64_t seed) {
  Rng R(seed);
  Handle* h = new Handle;
  Grid G = tower_grid(wx, wy, storeys, R);
  G.ox = ox;
  G.oy = oy;
  G.mat = uint8_t(m->id);
  fragment(G, MatProps{m->rho, m->ft, m->fb, m->fc, m->coh, m->mu}, R, h->g);
  return h;
}

// A city block: towers on a grid of lots, heights uniform in [smin, smax] storeys, each tower's
// material drawn from `mats` (n_mats entries).
void* svxs_city(int32_t lots_x, int32_t lots_y, int32_t smin, int32_t smax, int32_t wmin, int32_t wmax,
                const svxs_material* mats, int32_t n_mats, uint64_t seed) {
  Rng R(seed);
  Handle* h = new Handle;
  const double lot = (wmax + 4) * kVoxel;
  for (int32_t j = 0; j < lots_y; ++j)
    for (int32_t i = 0; i < lots_x; ++i) {
      const int wx = int(R.integer(wmin, wmax)), wy = int(R.integer(wmin, wmax));
      const int st = int(R.integer(smin, smax));
      const svxs_material& m = mats[size_t(R.integer(0, n_mats - 1))];
      Grid G = tower_grid(wx, wy, st, R);
      G.ox = i * lot;
      G.oy = j * lot;
      G.mat = uint8_t(m.id);
      fragment(G, MatProps{m.rho, m.ft, m.fb, m.fc, m.coh, m.mu}, R, h->g);
    }
  return h;
}

// A loose piece: a random connected cluster of about `voxels` voxels, ground-supported or free
// (inertial relief, nearest-centre node pinned), with an impact force of magnitude `impact` (N)
// on a seeded fragment.
void* svxs_piece(int64_t voxels, int32_t free_body_, double impact, const svxs_material* m, uint64_t seed) {
  Rng R(seed);
  Handle* h = new Handle;
  Grid G = blob_grid(std::max<int64_t>(voxels, 8), R);
  G.mat = uint8_t(m->id);
  G.grounded = !free_body_;
  fragment(G, MatProps{m->rho, m->ft, m->fb, m->fc, m->coh, m->mu}, R, h->g);
  const int32_t n = int32_t(h->g.nodes.size());
  int32_t node = n > 0 ? int32_t(R.integer(0, n - 1)) : -1;
  const double th = R.uniform(0, 6.283185307179586), ph = R.uniform(-1.0, 1.0);
  const double s = std::sqrt(std::max(0.0, 1.0 - ph * ph));
  const double F[3] = {impact * s * std::cos(th), impact * s * std::sin(th), impact * ph};
  if (free_body_) {
    free_body(h->g, 0, node, F);
  } else if (node >= 0) {
    for (int a = 0; a < 3; ++a) h->g.f[6 * size_t(node) + a] += F[a];
  }
  return h;
}

int32_t svxs_num_nodes(void* hp) { return int32_t(static_cast<Handle*>(hp)->g.nodes.size()); }
int32_t svxs_num_bonds(void* hp) { return int32_t(static_cast<Handle*>(hp)->g.bonds.size()); }

void svxs_get(void* hp, svxg_node* nodes, svxg_bond* bonds, double* f) {
  const Graph& g = static_cast<Handle*>(hp)->g;
  if (nodes) std::memcpy(nodes, g.nodes.data(), sizeof(svxg_node) * g.nodes.size());
  if (bonds) std::memcpy(bonds, g.bonds.data(), sizeof(svxg_bond) * g.bonds.size());
  if (f) std::memcpy(f, g.f.data(), sizeof(double) * g.f.size());
}

int32_t svxs_num_sections(void* hp) { return int32_t(static_cast<Handle*>(hp)->g.secs.size()); }
int64_t svxs_num_faces(void* hp) { return int64_t(static_cast<Handle*>(hp)->g.faces.size()); }

void svxs_get_sections(void* hp, svxg_section* secs, svxg_face* faces) {
  const Graph& g = static_cast<Handle*>(hp)->g;
  if (secs) std::memcpy(secs, g.secs.data(), sizeof(svxg_section) * g.secs.size());
  if (faces) std::memcpy(faces, g.faces.data(), sizeof(svxg_face) * g.faces.size());
}

void svxs_free(void* hp) { delete static_cast<Handle*>(hp); }

}  // extern "C"
