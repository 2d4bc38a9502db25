// svxg_svx.hpp - the reference-side binding: svx::GpuStressProblem, svx::StressProblem's
// interface (core/include/svx/stress/stress.hpp:74-160) over this library, in the reference's own
// types (SNode, SBond, MaterialTable, StressOptions, PcgResult, BondLoad), and the world's load
// builders on svx::Body.
//
// Built inside the reference's tree: it needs the reference's include directory
// (svx/stress/stress.hpp, svx/phys/rigid.hpp) and this repository's include/, and links
// libsvxg.so. World::Impl's Structure::P and BodyGraph::P (core/src/world/world_internal.hpp:745,
// :768) switch to it with `GpuStressProblem P;`: every member the world calls is here, with the
// same meaning, and like the reference it throws nothing (built with -fno-exceptions).
//
// Records are converted field by field (SBond keeps `sectioned` after `strength`, svxg_bond
// before it). The graph is taken from `nodes` / `bonds` / `mats` by every call that reads it
// (assemble, reassemble, solve, begin, extend_warm_start); flags the library changes (in_k,
// broken, gone) are written back. bond_load() serves the loads of the last u it was asked for
// (one device pass per distinct u) from the graph the last of those calls took.
#pragma once

#include <cmath>
#include <vector>

#include "svx/phys/rigid.hpp"
#include "svx/stress/stress.hpp"
#include "svxg_stress_problem.hpp"

namespace svx {

static_assert(kMaxMaterials == SVXG_MAX_MATERIALS, "material id ranges");
static_assert(sizeof(MaterialId) == 1, "material ids are bytes on both sides");

inline svxg_v3 to_svxg(const V3& v) { return svxg_v3{v.x, v.y, v.z}; }
inline V3 from_svxg(const svxg_v3& v) { return V3{v.x, v.y, v.z}; }

inline svxg_node to_svxg(const SNode& s) {
  svxg_node n{};
  n.c = to_svxg(s.c);
  n.mass = s.mass;
  n.fixed = s.fixed ? 1 : 0;
  n.gone = s.gone ? 1 : 0;
  return n;
}

inline svxg_bond to_svxg(const SBond& s) {
  svxg_bond b{};
  b.a = s.a;
  b.b = s.b;
  b.broken = s.broken ? 1 : 0;
  b.in_k = s.in_k ? 1 : 0;
  b.ma = static_cast<uint8_t>(s.ma);
  b.mb = static_cast<uint8_t>(s.mb);
  b.sectioned = s.sectioned ? 1 : 0;
  b.n = to_svxg(s.n);
  b.t1 = to_svxg(s.t1);
  b.t2 = to_svxg(s.t2);
  b.area = s.area;
  b.p = to_svxg(s.p);
  b.s1 = s.s1;
  b.s2 = s.s2;
  b.c1 = s.c1;
  b.c2 = s.c2;
  b.rmax = s.rmax;
  b.la = s.la;
  b.lb = s.lb;
  b.strength = s.strength;
  b.ft = s.ft;
  b.fb = s.fb;
  b.fc = s.fc;
  b.coh = s.coh;
  b.mu = s.mu;
  b.faces = s.faces;
  b.tag = s.tag;
  return b;
}

// every id's resolved properties (MaterialTable::operator[]: unregistered ids read id 0's)
inline std::vector<svxg_material> to_svxg(const MaterialTable& t) {
  std::vector<svxg_material> m(SVXG_MAX_MATERIALS);
  for (int i = 0; i < SVXG_MAX_MATERIALS; ++i) {
    const Material& x = t[static_cast<MaterialId>(i)];
    m[size_t(i)] = svxg_material{x.E, x.G, x.rho, x.ft, x.fb, x.fc, x.cohesion, x.friction};
  }
  return m;
}

inline svxg_amg_options to_svxg(const AmgOptions& o) {
  svxg_amg_options a{};
  a.coarse_max = o.coarse_max;
  a.smoothed = o.smoothed ? 1 : 0;
  a.strength = o.strength;
  a.coarse_scale = o.coarse_scale;
  a.max_levels = o.max_levels;
  a.gamma = o.gamma;
  a.sgs = o.sgs ? 1 : 0;
  a.sweeps = o.sweeps;
  a.cheb_degree = o.cheb_degree;
  a.dense_work_per_unknown = o.dense_work_per_unknown ? 1 : 0;
  a.coarsen_dense = o.coarsen_dense ? 1 : 0;
  a.reaggregate = o.reaggregate ? 1 : 0;
  return a;
}

inline svxg_stress_options to_svxg(const StressOptions& o, int32_t precision) {
  svxg_stress_options s = svxg_default_options();
  s.rtol = o.rtol;
  s.amg = to_svxg(o.amg);
  s.amg_min_nodes = o.amg_min_nodes;
  s.precision = precision;
  return s;
}

inline PcgResult from_svxg(const svxg_pcg_result& r) {
  PcgResult p;
  p.iters = r.iters;
  p.rel_res = r.rel_res;
  p.converged = r.converged != 0;
  p.breakdown = r.breakdown != 0;
  return p;
}

inline BondLoad from_svxg(const svxg_bond_load& L) {
  BondLoad b;
  b.N = L.N;
  b.V1 = L.V1;
  b.V2 = L.V2;
  b.T = L.T;
  b.M1 = L.M1;
  b.M2 = L.M2;
  return b;
}

inline svxg_bond_load to_svxg(const BondLoad& L) { return svxg_bond_load{L.N, L.V1, L.V2, L.T, L.M1, L.M2}; }

class GpuStressProblem {
 public:
  std::vector<SNode> nodes;
  std::vector<SBond> bonds;
  const MaterialTable* mats = nullptr;  // (nullptr: the process's, default_materials())
  // SVXG_PRECISION_*: FP64 (the reference's arithmetic) or the mixed-precision policy
  int32_t precision = SVXG_PRECISION_FP64;

  explicit GpuStressProblem(int device = 0) : g_(device) {}
  const MaterialTable& materials() const { return mats ? *mats : default_materials(); }
  bool ok() const { return g_.ok(); }
  const std::string& error() const { return g_.error(); }

  bool assemble(const StressOptions& opt = {}) {
    take();
    const bool r = g_.assemble(to_svxg(opt, precision));
    give();
    return r;
  }
  bool assembled() const { return g_.assembled(); }
  void invalidate() { g_.invalidate(); }
  bool preconditioner_current() const { return g_.preconditioner_current(); }
  bool block_jacobi() const { return g_.block_jacobi(); }
  i64 assembly_work() const { return g_.assembly_work(); }
  void release() {
    g_.release();
    give();
  }
  void remove_bond(i32 b) {
    if (b < 0 || size_t(b) >= bonds.size()) return;
    g_.remove_bond(b);
    give();
  }
  void retire_nodes(const std::vector<i32>& list) {
    g_.retire_nodes(list);
    give();
  }
  bool reassemble() {
    take();
    const bool r = g_.reassemble();
    give();
    return r;
  }
  void extend_warm_start(std::vector<f64>& u, i32 first_new_node) const {
    take();
    g_.extend_warm_start(u, first_new_node);
  }
  i32 appended() const { return g_.appended(); }
  i32 free_nodes() const { return g_.free_nodes(); }
  i64 matrix_blocks() const { return g_.matrix_blocks(); }
  i64 memory_bytes(Bytes kind = Bytes::Held) const {
    const svxg::Bytes k = kind == Bytes::Held ? svxg::Bytes::Held : svxg::Bytes::Used;
    const auto own = [&](const auto& v) { return i64((kind == Bytes::Held ? v.capacity() : v.size()) * sizeof(v[0])); };
    return own(nodes) + own(bonds) + g_.memory_bytes(k);
  }
  i64 solver_bytes(Bytes kind = Bytes::Held) const {
    return g_.solver_bytes(kind == Bytes::Held ? svxg::Bytes::Held : svxg::Bytes::Used);
  }
  i64 work_per_iteration() const { return g_.work_per_iteration(); }

  PcgResult solve(const std::vector<f64>& f, std::vector<f64>& u, f64 rtol, int maxit, bool warm) {
    take();
    const PcgResult r = from_svxg(g_.solve(f, u, rtol, maxit, warm));
    give();
    return r;
  }
  void begin(const std::vector<f64>& f, const std::vector<f64>& u0) {
    take();
    g_.begin(f, u0);
  }
  PcgResult iterate(int maxit, f64 rtol) { return from_svxg(g_.iterate(maxit, rtol)); }
  bool running() const { return g_.running(); }
  void stop() { g_.stop(); }
  void current(std::vector<f64>& u) const { g_.current(u); }
  BondLoad bond_load(i32 b, const std::vector<f64>& u) const { return from_svxg(g_.bond_load(b, u)); }
  static void add_force(std::vector<f64>& f, i32 node, const V3& c, const V3& F, const V3& at) {
    svxg::StressProblem::add_force(f, node, to_svxg(c), to_svxg(F), to_svxg(at));
  }

  // the library's own members: the device judge of every bond, the break rounds, counters
  svxg::StressProblem& device() { return g_; }
  const svxg::StressProblem& device() const { return g_; }

 private:
  // the graph as the caller left it, into the library's records (the library uploads it only
  // when its contents changed since the last upload)
  void take() const {
    g_.nodes.resize(nodes.size());
    for (size_t i = 0; i < nodes.size(); ++i) g_.nodes[i] = to_svxg(nodes[i]);
    g_.bonds.resize(bonds.size());
    for (size_t k = 0; k < bonds.size(); ++k) g_.bonds[k] = to_svxg(bonds[k]);
    g_.mats = to_svxg(materials());
  }
  // the flags the library keeps (stress.hpp: in_k by assemble, broken by remove_bond, gone and
  // broken by retire_nodes)
  void give() {
    for (size_t i = 0; i < nodes.size() && i < g_.nodes.size(); ++i) nodes[i].gone = g_.nodes[i].gone != 0;
    for (size_t k = 0; k < bonds.size() && k < g_.bonds.size(); ++k) {
      bonds[k].broken = g_.bonds[k].broken != 0;
      bonds[k].in_k = g_.bonds[k].in_k != 0;
    }
  }
  mutable svxg::StressProblem g_;
};

// The world's loads in its own types. A structure's: weight per node down z plus ext (6 per node,
// may be empty) - World::Impl::load_vector (core/src/world/world.cpp:966-974).
inline std::vector<f64> gpu_load_vector(const std::vector<f64>& weight, const std::vector<f64>& ext) {
  return svxg::load_vector(weight, ext);
}

// A free piece's pinned node - pin_reference (core/src/world/world_pieces.cpp:313-326).
inline i32 gpu_pin_reference(std::vector<SNode>& nodes, const V3& com) {
  i32 pin = -1;
  std::vector<svxg_node> n(nodes.size());
  for (size_t i = 0; i < nodes.size(); ++i) n[i] = to_svxg(nodes[i]);
  pin = svxg_pin_reference(n.data(), i32(n.size()), to_svxg(com));
  for (size_t i = 0; i < nodes.size(); ++i) nodes[i].fixed = n[i].fixed != 0;
  return pin;
}

// A moving piece's loads - World::Impl::body_stress_run (world_pieces.cpp:566-603): the graph's
// per-node centre (body frame), mass and inertia (BodyGraph::node_com / node_mass / node_inertia),
// and the point forces with the node each acts on (the world's frag_node of PointForce::frag;
// -1: none).
struct GpuPointForce {
  i32 node;
  V3 F, p;
};
inline std::vector<f64> gpu_body_loads(const Body& b, f64 gravity, const std::vector<SNode>& nodes,
                                       const std::vector<V3>& node_com, const std::vector<f64>& node_mass,
                                       const std::vector<M3>& node_inertia,
                                       const std::vector<GpuPointForce>& forces, bool inertia) {
  svxg_body_state s{};
  s.x = to_svxg(b.x);
  s.q[0] = b.q.x;
  s.q[1] = b.q.y;
  s.q[2] = b.q.z;
  s.q[3] = b.q.w;
  s.com = to_svxg(b.com);
  s.w = to_svxg(b.w);
  for (int k = 0; k < 9; ++k) {
    s.inertia[k] = b.inertia.m[size_t(k)];
    s.inv_inertia[k] = b.inv_inertia.m[size_t(k)];
  }
  s.inv_mass = b.inv_mass;
  s.gravity = gravity;
  std::vector<svxg_node> n(nodes.size());
  for (size_t i = 0; i < nodes.size(); ++i) n[i] = to_svxg(nodes[i]);
  std::vector<svxg_v3> com(node_com.size());
  for (size_t i = 0; i < node_com.size(); ++i) com[i] = to_svxg(node_com[i]);
  std::vector<f64> I(9 * node_inertia.size());
  for (size_t i = 0; i < node_inertia.size(); ++i)
    for (int k = 0; k < 9; ++k) I[9 * i + size_t(k)] = node_inertia[i].m[size_t(k)];
  std::vector<svxg_point_force> pf(forces.size());
  for (size_t k = 0; k < forces.size(); ++k) pf[k] = svxg_point_force{to_svxg(forces[k].F), to_svxg(forces[k].p), forces[k].node, 0};
  return svxg::body_loads(s, n, com, node_mass, I, pf, inertia);
}

}  // namespace svx
