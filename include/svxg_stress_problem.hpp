// svxg_stress_problem.hpp - C++20 host class with svx::StressProblem's interface over the C ABI.
//
// The reference's callers hold a `StressProblem` (core/include/svx/stress/stress.hpp:74-160):
// public `nodes`, `bonds`, `mats`, then assemble / solve / begin / iterate / current /
// bond_load / remove_bond / retire_nodes / release and the work counters. This class keeps that
// shape over include/svxg.h so a host written against the reference reads the same; every number
// comes from the CUDA library. Records are svxg_node / svxg_bond (byte images of SNode / SBond,
// include/svxg_types.h); `mats` is a table of SVXG_MAX_MATERIALS resolved entries.
//
// Like the reference, callers may change `nodes` and `bonds` between calls: the graph is sent to
// the device at assemble(), and again before a solve when its contents changed since (which, as
// assembling again would, drops the assembled operator).
//
// Errors follow the reference's contract, which is built without exceptions (CMakeLists.txt:248,
// -fno-exceptions): nothing here throws. A failed library call leaves its message in error()
// (and svxg_last_error()); assemble() then returns false, solve() / iterate() a result with
// breakdown set and rel_res = inf (the reference's answer for an unassembled problem,
// stress.cpp:349-354), and the other members leave their outputs empty or zero. A problem whose
// device could not be set up (ok() false) fails every call that way.
#pragma once

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "svxg.h"

namespace svxg {

// What a byte count counts (svx::Bytes, core/include/svx/base/mem.hpp:14): Held - what the
// problem holds (host vectors' capacities, device allocations); Used - what it uses (host vectors'
// elements; the device side is allocated to size, so both count the same there).
enum class Bytes : uint8_t { Held, Used };

class StressProblem {
 public:
  std::vector<svxg_node> nodes;
  std::vector<svxg_bond> bonds;
  std::vector<svxg_material> mats;  // SVXG_MAX_MATERIALS entries

  explicit StressProblem(int device = 0) {
    if (svxg_problem_create(&p_, device) != SVXG_OK) {
      p_ = nullptr;
      note_error();
    }
  }
  ~StressProblem() {
    if (p_) svxg_problem_destroy(p_);
  }
  StressProblem(const StressProblem&) = delete;
  StressProblem& operator=(const StressProblem&) = delete;

  // whether the device side exists; the message of the last failed call
  bool ok() const { return p_ != nullptr; }
  const std::string& error() const { return error_; }

  // stress.hpp:83 - K and the preconditioner; false on a singular diagonal or a failed call
  bool assemble(const svxg_stress_options& opt = svxg_default_options()) {
    if (!upload()) return false;
    int32_t ok = 0;
    if (!check(svxg_assemble(p_, &opt, &ok))) return false;
    pull_flags();
    return ok != 0;
  }
  bool assembled() const { return p_ && svxg_assembled(p_) == 1; }
  void invalidate() { check(svxg_invalidate(p_)); }
  bool preconditioner_current() const { return p_ && svxg_preconditioner_current(p_) == 1; }
  bool block_jacobi() const { return p_ && svxg_block_jacobi(p_) == 1; }
  int64_t assembly_work() const { return info().assembly_work; }
  void release() {
    if (!check(svxg_release(p_))) return;
    for (auto& b : bonds) b.in_k = 0;
    sent_bonds_ = bonds;
    ++generation_;
  }
  void remove_bond(int32_t b) {
    if (check(svxg_remove_bond(p_, b))) pull_flags();
  }
  void retire_nodes(const std::vector<int32_t>& list) {
    if (!check(svxg_retire_nodes(p_, list.data(), int32_t(list.size())))) return;
    for (int32_t i : list) nodes[size_t(i)].gone = 1;
    sent_nodes_ = nodes;
    pull_flags();
  }
  // stress.hpp:110 - K again from nodes and bonds as they are now; appended nodes get their own
  // preconditioner, the old one keeps the rest
  bool reassemble() {
    if (!mats_complete()) return false;
    int32_t ok = 0;
    if (!check(svxg_reassemble(p_, nodes.data(), int32_t(nodes.size()), bonds.data(), int32_t(bonds.size()),
                               mats.data(), &ok)))
      return false;
    sent_nodes_ = nodes;
    sent_bonds_ = bonds;
    pull_flags();
    return ok != 0;
  }
  // stress.hpp:113 - appended nodes' warm start from their older neighbours (u: 6 per node)
  void extend_warm_start(std::vector<double>& u, int32_t first_new_node) const {
    if (!upload_if_changed() || u.size() != 6 * nodes.size()) return;
    check(svxg_extend_warm_start(p_, u.data(), first_new_node));
  }
  int32_t appended() const { return p_ ? svxg_appended(p_) : 0; }
  int32_t free_nodes() const { return info().nfree; }
  int64_t matrix_blocks() const { return info().matrix_blocks; }
  // stress.hpp:116-117 - the graph's records and the solver; of those, what release() frees
  int64_t memory_bytes(Bytes kind = Bytes::Held) const {
    const svxg_info i = info();
    return host_bytes(nodes, kind) + host_bytes(bonds, kind) + host_bytes(mats, kind) + i.device_bytes;
  }
  int64_t solver_bytes(Bytes kind = Bytes::Held) const {
    (void)kind;
    const svxg_info i = info();
    return i.device_bytes - i.graph_bytes;
  }
  int64_t work_per_iteration() const { return info().work_per_iteration; }

  // stress.hpp:122 - f, u: 6 per node; u: warm start in, solution out; maxit < 0: no cap
  svxg_pcg_result solve(const std::vector<double>& f, std::vector<double>& u, double rtol, int maxit, bool warm) {
    u.resize(6 * nodes.size(), 0.0);
    if (f.size() != 6 * nodes.size()) {
      error_ = "svxg: f needs 6 entries per node";
      return failed();
    }
    if (!upload_if_changed()) return failed();
    svxg_pcg_result r{};
    if (!check(svxg_solve(p_, f.data(), u.data(), rtol, maxit, warm ? 1 : 0, &r))) return failed();
    pull_flags();
    return r;
  }
  void begin(const std::vector<double>& f, const std::vector<double>& u0) {
    if (f.size() != 6 * nodes.size()) {
      error_ = "svxg: f needs 6 entries per node";
      return;
    }
    if (!upload_if_changed()) return;
    check(svxg_begin(p_, f.data(), u0.size() == 6 * nodes.size() ? u0.data() : nullptr));
  }
  svxg_pcg_result iterate(int maxit, double rtol) {
    svxg_pcg_result r{};
    if (!check(svxg_iterate(p_, maxit, rtol, &r))) return failed();
    return r;
  }
  bool running() const { return p_ && svxg_running(p_) == 1; }
  void stop() { check(svxg_stop(p_)); }
  void current(std::vector<double>& u) const {
    u.assign(6 * nodes.size(), 0.0);
    check(svxg_current(p_, u.data()));
  }

  // stress.hpp:132 - one bond's load at u. The reference's callers ask bond by bond at one u
  // (world.cpp:1174, :1238, :1927; world_io.cpp:98, :122); the device evaluates every bond at once,
  // so the loads of the last u asked for are kept here and served while the two nodes a bond reads
  // (u of its ends) are unchanged and no call changed the graph since: one device pass per
  // distinct u, O(1) host work per call. Changes callers make to `nodes` / `bonds` themselves are
  // seen by the next device pass (a new u, or bond_loads()).
  svxg_bond_load bond_load(int32_t b, const std::vector<double>& u) const {
    if (b < 0 || size_t(b) >= bonds.size() || u.size() != 6 * nodes.size()) return svxg_bond_load{};
    if (!cache_serves(b, u)) {
      cache_.loads = bond_loads(u);
      cache_.u = u;
      cache_.generation = generation_;
      cache_.valid = cache_.loads.size() == bonds.size();
      ++cache_.device_passes;
      if (!cache_.valid) return svxg_bond_load{};
    }
    return cache_.loads[size_t(b)];
  }
  // every bond's load at u, one device pass
  std::vector<svxg_bond_load> bond_loads(const std::vector<double>& u) const {
    if (u.size() != 6 * nodes.size() || !upload_if_changed()) return {};
    std::vector<svxg_bond_load> out(bonds.size());
    if (!check(svxg_bond_loads(p_, u.data(), out.data()))) return {};
    return out;
  }
  // device passes bond_load() has made (for callers checking the per-u cache)
  int64_t bond_load_passes() const { return cache_.device_passes; }
  // bond_utilization (stress.hpp:64-66) of every bond at the current solution; failing bonds
  struct Judgement {
    std::vector<double> phi;
    std::vector<uint8_t> mode;
    std::vector<int32_t> failing;
  };
  Judgement judge(double fragility) const {
    Judgement j;
    j.phi.resize(bonds.size());
    j.mode.resize(bonds.size());
    j.failing.resize(bonds.size() + 1);
    int32_t n = 0;
    if (!check(svxg_utilization(p_, fragility, j.phi.data(), j.mode.data(), j.failing.data(),
                                int32_t(j.failing.size()), &n)))
      return Judgement{};
    j.failing.resize(size_t(n));
    return j;
  }

  // stress.hpp:134 - a force F at point `at` on a node with centre c
  static void add_force(std::vector<double>& f, int32_t node, svxg_v3 c, svxg_v3 F, svxg_v3 at) {
    double* fi = &f[6 * size_t(node)];
    fi[0] += F.x;
    fi[1] += F.y;
    fi[2] += F.z;
    const double rx = at.x - c.x, ry = at.y - c.y, rz = at.z - c.z;
    fi[3] += ry * F.z - rz * F.y;
    fi[4] += rz * F.x - rx * F.z;
    fi[5] += rx * F.y - ry * F.x;
  }

  // World::Impl::judge's break rounds of this structure (svxg_cascade): nodes and bonds are left
  // retired and broken as the reference's world leaves them. judged / judged_has: the steady loads
  // per bond, in and out (both empty: none yet; then they are filled).
  struct Cascade {
    svxg_cascade_result result{};
    std::vector<int32_t> broken, retired;
    std::vector<double> phi;
  };
  Cascade cascade(const std::vector<double>& f, std::vector<double>& u,
                  const svxg_cascade_options& o = svxg_default_cascade_options(),
                  std::vector<svxg_bond_load>* judged = nullptr, std::vector<uint8_t>* judged_has = nullptr) {
    Cascade c;
    u.resize(6 * nodes.size(), 0.0);
    if (f.size() != 6 * nodes.size() || !upload_if_changed()) {
      c.result.status = SVXG_ERR_ARG;
      return c;
    }
    c.broken.resize(bonds.size() + 1);
    c.retired.resize(nodes.size() + 1);
    c.phi.resize(bonds.size() + 1);
    if (judged && judged_has) {
      judged->resize(bonds.size());
      judged_has->resize(bonds.size(), 0);
    }
    const int e = svxg_cascade(p_, nullptr, &o, f.data(), u.data(), judged && judged_has ? judged->data() : nullptr,
                               judged && judged_has ? judged_has->data() : nullptr, c.phi.data(), c.broken.data(),
                               int32_t(c.broken.size()), c.retired.data(), int32_t(c.retired.size()), &c.result);
    if (!check(e)) {
      c = Cascade{};
      c.result.status = e;
      return c;
    }
    c.broken.resize(size_t(c.result.bonds_broken));
    c.retired.resize(size_t(c.result.nodes_retired));
    c.phi.resize(bonds.size());
    for (int32_t i : c.retired) nodes[size_t(i)].gone = 1;
    sent_nodes_ = nodes;
    pull_flags();
    return c;
  }

  // World::Impl::body_stress_run's break rounds of this piece (svxg_piece_rounds): f is its load
  // and comes back with the chips' loads moved; gf: fracture energy per material (null: presets).
  struct PieceRounds {
    svxg_piece_result result{};
    std::vector<int32_t> broken, chips;
    std::vector<uint8_t> modes;
  };
  PieceRounds piece_rounds(std::vector<double>& f, std::vector<double>& u,
                           const svxg_piece_options& o = svxg_default_piece_options(), const double* gf = nullptr) {
    PieceRounds r;
    u.resize(6 * nodes.size(), 0.0);
    if (f.size() != 6 * nodes.size() || !upload_if_changed()) {
      r.result.status = SVXG_ERR_ARG;
      return r;
    }
    r.broken.resize(bonds.size() + 1);
    r.modes.resize(bonds.size() + 1);
    r.chips.resize(nodes.size() + 1);
    const int e = svxg_piece_rounds(p_, nullptr, &o, gf, f.data(), u.data(), r.broken.data(), r.modes.data(),
                                    int32_t(r.broken.size()), r.chips.data(), int32_t(r.chips.size()), &r.result);
    if (!check(e)) {
      r = PieceRounds{};
      r.result.status = e;
      return r;
    }
    r.broken.resize(size_t(r.result.bonds_broken));
    r.modes.resize(size_t(r.result.bonds_broken));
    r.chips.resize(size_t(r.result.chips));
    for (int32_t i : r.chips) nodes[size_t(i)].gone = 1;
    sent_nodes_ = nodes;
    pull_flags();
    return r;
  }

  svxg_info info() const {
    svxg_info i{};
    check(svxg_get_info(p_, &i));
    return i;
  }
  svxg_problem* handle() const { return p_; }

 private:
  // false (and the message kept) for a failed call; a missing device side fails every call
  bool check(int code) const {
    if (!p_) {
      if (error_.empty()) error_ = "svxg: no device problem";
      return false;
    }
    if (code >= 0) return true;
    note_error();
    return false;
  }
  void note_error() const { error_ = std::string("svxg: ") + svxg_last_error(); }
  static svxg_pcg_result failed() {
    svxg_pcg_result r{};
    r.breakdown = 1;
    r.rel_res = INFINITY;
    return r;
  }
  bool mats_complete() const {
    if (mats.size() == SVXG_MAX_MATERIALS) return true;
    error_ = "svxg: mats needs every material id";
    return false;
  }
  template <class T>
  static int64_t host_bytes(const std::vector<T>& v, Bytes kind) {
    return int64_t((kind == Bytes::Held ? v.capacity() : v.size()) * sizeof(T));
  }
  bool upload() const {
    if (!mats_complete()) return false;
    if (!check(svxg_set_graph(p_, nodes.data(), int32_t(nodes.size()), bonds.data(), int32_t(bonds.size()),
                              mats.data())))
      return false;
    sent_nodes_ = nodes;
    sent_bonds_ = bonds;
    ++generation_;
    return true;
  }
  static bool same(const void* a, const void* b, size_t n) { return n == 0 || std::memcmp(a, b, n) == 0; }
  bool upload_if_changed() const {
    if (nodes.size() != sent_nodes_.size() || bonds.size() != sent_bonds_.size() ||
        !same(nodes.data(), sent_nodes_.data(), nodes.size() * sizeof(svxg_node)) ||
        !same(bonds.data(), sent_bonds_.data(), bonds.size() * sizeof(svxg_bond)))
      return upload();
    return true;
  }
  void pull_flags() {
    std::vector<uint8_t> br(bonds.size()), ik(bonds.size());
    ++generation_;
    if (!check(svxg_bond_flags(p_, br.data(), ik.data()))) return;
    for (size_t k = 0; k < bonds.size(); ++k) {
      bonds[k].broken = br[k];
      bonds[k].in_k = ik[k];
    }
    sent_bonds_ = bonds;
  }
  // the per-u loads serve bond b while the graph is the one they were made from and u is the
  // same at b's ends (a bond's load reads u at its two nodes only, stress.cpp:477-502)
  bool cache_serves(int32_t b, const std::vector<double>& u) const {
    if (!cache_.valid || cache_.generation != generation_ || cache_.u.size() != u.size()) return false;
    const svxg_bond& bd = bonds[size_t(b)];
    if (bd.a < 0 || size_t(bd.a) >= nodes.size()) return false;
    if (!same(&u[6 * size_t(bd.a)], &cache_.u[6 * size_t(bd.a)], 6 * sizeof(double))) return false;
    if (bd.b >= 0 && (size_t(bd.b) >= nodes.size() ||
                      !same(&u[6 * size_t(bd.b)], &cache_.u[6 * size_t(bd.b)], 6 * sizeof(double))))
      return false;
    return true;
  }
  struct LoadCache {
    bool valid = false;
    uint64_t generation = 0;
    int64_t device_passes = 0;
    std::vector<double> u;
    std::vector<svxg_bond_load> loads;
  };
  svxg_problem* p_ = nullptr;
  // (the device's copy of the graph is state behind const members too, as the reference's
  // bond_load and extend_warm_start read the public members as they are)
  mutable std::vector<svxg_node> sent_nodes_;
  mutable std::vector<svxg_bond> sent_bonds_;
  mutable uint64_t generation_ = 0;
  mutable LoadCache cache_;
  mutable std::string error_;
};

// SecAcc::finish + section_strengths(_general) of every interface (svxg_build_bonds): bond k of
// the result from secs[k].
inline std::vector<svxg_bond> build_bonds(const std::vector<svxg_node>& nodes, const std::vector<svxg_section>& secs,
                                          const std::vector<svxg_face>& faces,
                                          const std::vector<svxg_material>& mats,
                                          const std::vector<svxg_junction>& junctions = {},
                                          const std::vector<svxg_lattice>& lattices = {}, int32_t samples = 2) {
  std::vector<svxg_bond> out(secs.size());
  const int e = svxg_build_bonds(nodes.data(), int32_t(nodes.size()), secs.data(), int32_t(secs.size()), faces.data(),
                                 int64_t(faces.size()), junctions.empty() ? nullptr : junctions.data(),
                                 int64_t(junctions.size()), lattices.empty() ? nullptr : lattices.data(),
                                 int32_t(lattices.size()), samples, mats.data(), out.data());
  if (e < 0) return {};  // (the message: svxg_last_error())
  return out;
}

// bond_strength / bond_utilization (stress.hpp:53-66): the reference's free functions, the same
// arithmetic as the device judge. strength: {ft, fb, fc, cohesion, friction}; a bad material id
// gives phi -1 and an empty strength.
inline std::vector<double> bond_strength(const svxg_bond& b, double fragility, const std::vector<svxg_material>& mats) {
  std::vector<double> s(5);
  if (mats.size() < SVXG_MAX_MATERIALS || svxg_bond_strength(&b, fragility, mats.data(), s.data()) != SVXG_OK) return {};
  return s;
}
inline double bond_utilization(const svxg_bond& b, const svxg_bond_load& L, double fragility,
                               const std::vector<svxg_material>& mats, uint8_t* mode = nullptr) {
  if (mats.size() < SVXG_MAX_MATERIALS) return -1.0;
  return svxg_bond_utilization(&b, &L, fragility, mats.data(), mode);
}

// The world's loads (svxg_structure_loads, svxg_pin_reference, svxg_body_loads): a structure's
// load vector (World::Impl::load_vector, world.cpp:966-974), a free piece's pinned node
// (pin_reference, world_pieces.cpp:313-326) and a moving piece's loads (world_pieces.cpp:566-603).
inline std::vector<double> load_vector(const std::vector<double>& weight, const std::vector<double>& ext = {}) {
  std::vector<double> f(6 * weight.size());
  if (!ext.empty() && ext.size() != f.size()) return {};
  if (svxg_structure_loads(int32_t(weight.size()), weight.data(), ext.empty() ? nullptr : ext.data(), f.data()) !=
      SVXG_OK)
    return {};
  return f;
}
inline int32_t pin_reference(std::vector<svxg_node>& nodes, svxg_v3 com) {
  return svxg_pin_reference(nodes.data(), int32_t(nodes.size()), com);
}
// node_inertia: 9 per node (body frame, about node_com); forces name their node (-1: none)
inline std::vector<double> body_loads(const svxg_body_state& b, const std::vector<svxg_node>& nodes,
                                      const std::vector<svxg_v3>& node_com, const std::vector<double>& node_mass,
                                      const std::vector<double>& node_inertia,
                                      const std::vector<svxg_point_force>& forces, bool inertia) {
  const size_t n = nodes.size();
  if (inertia && (node_com.size() != n || node_mass.size() != n || node_inertia.size() != 9 * n)) return {};
  std::vector<double> f(6 * n);
  if (svxg_body_loads(&b, nodes.data(), int32_t(n), inertia ? node_com.data() : nullptr,
                      inertia ? node_mass.data() : nullptr, inertia ? node_inertia.data() : nullptr, forces.data(),
                      int32_t(forces.size()), inertia ? 1 : 0, f.data()) != SVXG_OK)
    return {};
  return f;
}

}  // namespace svxg
