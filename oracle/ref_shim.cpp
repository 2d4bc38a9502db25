// ref_shim.cpp - TEST INFRASTRUCTURE ONLY (the oracle). Never part of the shipped library.
//
// A C ABI over the reference's own svx::StressProblem / svx::Amg, compiled together with the
// reference's solve sources (core/src/solve/amg.cpp, core/src/stress/stress.cpp,
// core/src/material/material.cpp, core/src/base/parallel.cpp) by oracle/build_oracle.py into
// oracle/_ref/libsvxref.so. The tests use it to pin the C restatement (oracle/svx_oracle.c) and to
// write the golden fixtures; bench.py's reference arm times it where it exists.
//
// The hierarchy export needs the multigrid's levels before Amg::make_fast frees their
// double-precision copies (core/src/solve/amg.cpp:594-628), so this file alone opens the
// reference classes' private members (the access keyword only: layouts are unchanged) and walks
// the build's level loop (core/src/solve/amg.cpp:285-304) itself.
#define private public
#include "svx/base/parallel.hpp"
#include "svx/material/material.hpp"
#include "svx/solve/amg.hpp"
#include "svx/stress/stress.hpp"
#undef private

#include <chrono>
#include <cstring>
#include <map>
#include <vector>

#include "world_internal.hpp"  // (SecAcc, section_strengths: header-only, core/src/world)

#include "svxg_types.h"

using namespace svx;

namespace {

static_assert(sizeof(svxg_node) == 40, "svxg_node layout");
static_assert(sizeof(svxg_bond) == 216, "svxg_bond layout");
static_assert(sizeof(svxg_material) == 64, "svxg_material layout");

V3 v3(const svxg_v3& v) { return V3{v.x, v.y, v.z}; }

void fill_materials(MaterialTable& t, const svxg_material* m) {
  for (int i = 0; i < SVXG_MAX_MATERIALS; ++i) {
    Material x = t[static_cast<MaterialId>(i)];
    x.E = m[i].E;
    x.G = m[i].G;
    x.rho = m[i].rho;
    x.ft = m[i].ft;
    x.fb = m[i].fb;
    x.fc = m[i].fc;
    x.cohesion = m[i].cohesion;
    x.friction = m[i].friction;
    t.set(static_cast<MaterialId>(i), x);
  }
}

void fill_problem(StressProblem& P, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb) {
  P.nodes.resize(size_t(n));
  for (int32_t i = 0; i < n; ++i) {
    SNode& s = P.nodes[size_t(i)];
    s.c = v3(nodes[i].c);
    s.mass = nodes[i].mass;
    s.fixed = nodes[i].fixed != 0;
    s.gone = nodes[i].gone != 0;
  }
  P.bonds.resize(size_t(nb));
  for (int32_t k = 0; k < nb; ++k) {
    const svxg_bond& b = bonds[k];
    SBond& s = P.bonds[size_t(k)];
    s.a = b.a;
    s.b = b.b;
    s.broken = b.broken != 0;
    s.in_k = b.in_k != 0;
    s.ma = static_cast<MaterialId>(b.ma);
    s.mb = static_cast<MaterialId>(b.mb);
    s.n = v3(b.n);
    s.t1 = v3(b.t1);
    s.t2 = v3(b.t2);
    s.area = b.area;
    s.p = v3(b.p);
    s.s1 = b.s1;
    s.s2 = b.s2;
    s.c1 = b.c1;
    s.c2 = b.c2;
    s.rmax = b.rmax;
    s.la = b.la;
    s.lb = b.lb;
    s.strength = b.strength;
    s.sectioned = b.sectioned != 0;
    s.ft = b.ft;
    s.fb = b.fb;
    s.fc = b.fc;
    s.coh = b.coh;
    s.mu = b.mu;
    s.faces = b.faces;
    s.tag = b.tag;
  }
}

StressOptions options(const svxg_stress_options* o) {
  StressOptions so;
  if (!o) return so;
  so.rtol = o->rtol;
  so.amg.coarse_max = o->amg.coarse_max;
  so.amg.strength = o->amg.strength;
  so.amg.smoothed = o->amg.smoothed != 0;
  so.amg.coarse_scale = o->amg.coarse_scale;
  so.amg.max_levels = o->amg.max_levels;
  so.amg.gamma = o->amg.gamma;
  so.amg.sgs = o->amg.sgs != 0;
  so.amg.sweeps = o->amg.sweeps;
  so.amg.cheb_degree = o->amg.cheb_degree;
  so.amg.dense_work_per_unknown = o->amg.dense_work_per_unknown != 0;
  so.amg.coarsen_dense = o->amg.coarsen_dense != 0;
  so.amg.reaggregate = o->amg.reaggregate != 0;
  so.amg_min_nodes = o->amg_min_nodes;
  return so;
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Hier {
  Amg amg;
  std::vector<f64> lmax;  // lambda_max(D^-1 A) estimate per level (the prolongation's damping)
};

}  // namespace

extern "C" {

struct svxr_info {
  int32_t nfree, levels, block_jacobi, chol_n;
  int32_t level_sizes[16];
  int64_t level_blocks[32];
  int64_t matrix_blocks, work_per_iteration, assembly_work, work_per_apply, build_work;
};

void svxr_set_threads(int n) { set_num_threads(n); }
int svxr_num_threads(void) { return num_threads(); }

// assemble() + solve() of the reference problem. u: 6 per node (warm start in, solution out).
// bonds[].in_k is written back. Returns assemble()'s result (1/0).
int svxr_solve(const svxg_node* nodes, int32_t n, svxg_bond* bonds, int32_t nb, const svxg_material* mats,
               const svxg_stress_options* o, const double* f, double* u, double rtol, int32_t maxit, int32_t warm,
               svxg_pcg_result* res, svxr_info* info, double* t_assemble, double* t_solve) {
  MaterialTable table;
  fill_materials(table, mats);
  StressProblem P;
  P.mats = &table;
  fill_problem(P, nodes, n, bonds, nb);
  const double t0 = now_s();
  const bool ok = P.assemble(options(o));
  const double t1 = now_s();
  std::vector<f64> fv(f, f + 6 * size_t(n)), uv(u, u + 6 * size_t(n));
  PcgResult r;
  double t2 = t1, t3 = t1;
  if (ok) {
    t2 = now_s();
    r = P.solve(fv, uv, rtol, maxit, warm != 0);
    t3 = now_s();
    std::memcpy(u, uv.data(), sizeof(double) * 6 * size_t(n));
  }
  if (res) {
    res->iters = r.iters;
    res->converged = r.converged;
    res->breakdown = r.breakdown;
    res->rel_res = r.rel_res;
  }
  for (int32_t k = 0; k < nb; ++k) bonds[k].in_k = P.bonds[size_t(k)].in_k ? 1 : 0;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->nfree = P.free_nodes();
    info->block_jacobi = P.block_jacobi();
    info->levels = P.amg_.levels();
    info->chol_n = P.amg_.chol_n_;
    const std::vector<i32> ls = P.amg_.level_sizes();
    const std::vector<i64> lb = P.amg_.level_blocks();
    for (size_t i = 0; i < ls.size() && i < 16; ++i) info->level_sizes[i] = ls[i];
    for (size_t i = 0; i < lb.size() && i < 32; ++i) info->level_blocks[i] = lb[i];
    info->matrix_blocks = P.matrix_blocks();
    info->work_per_iteration = P.work_per_iteration();
    info->assembly_work = P.assembly_work();
    info->work_per_apply = P.amg_.work_per_apply();
    info->build_work = P.amg_.build_work();
  }
  if (t_assemble) *t_assemble = t1 - t0;
  if (t_solve) *t_solve = t3 - t2;
  return ok ? 1 : 0;
}

// StressProblem::extend_warm_start (core/src/stress/stress.cpp:213-244) of u (6 per node, in
// and out) for nodes first_new and up.
void svxr_extend_warm_start(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                            const svxg_material* mats, double* u, int32_t first_new) {
  MaterialTable table;
  fill_materials(table, mats);
  StressProblem P;
  P.mats = &table;
  fill_problem(P, nodes, n, bonds, nb);
  std::vector<f64> uv(u, u + 6 * size_t(n));
  P.extend_warm_start(uv, first_new);
  std::memcpy(u, uv.data(), sizeof(double) * 6 * size_t(n));
}

// The judge's per-bond work: bond_load and bond_utilization (core/src/stress/stress.cpp:477-502,
// :23-57) of every bond at u (6 per node).
void svxr_judge(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb, const svxg_material* mats,
                const double* u, double fragility, svxg_bond_load* loads, double* phi, uint8_t* mode, double* t_judge) {
  MaterialTable table;
  fill_materials(table, mats);
  StressProblem P;
  P.mats = &table;
  fill_problem(P, nodes, n, bonds, nb);
  std::vector<f64> uv(u, u + 6 * size_t(n));
  const double t0 = now_s();
  for (int32_t k = 0; k < nb; ++k) {
    const BondLoad L = P.bond_load(k, uv);
    FailMode m = FailMode::None;
    const f64 ph = bond_utilization(P.bonds[size_t(k)], L, fragility, table, &m);
    if (loads) loads[k] = svxg_bond_load{L.N, L.V1, L.V2, L.T, L.M1, L.M2};
    if (phi) phi[k] = ph;
    if (mode) mode[k] = static_cast<uint8_t>(m);
  }
  if (t_judge) *t_judge = now_s() - t0;
}

// bond_utilization of given loads (the failure-mode known answers).
double svxr_utilization(const svxg_bond* bond, const svxg_bond_load* L, double fragility, const svxg_material* mats,
                        uint8_t* mode) {
  MaterialTable table;
  fill_materials(table, mats);
  StressProblem P;
  svxg_node dummy[2] = {};
  svxg_bond b = *bond;
  b.a = 0;
  b.b = b.b >= 0 ? 1 : -1;
  fill_problem(P, dummy, 2, &b, 1);
  BondLoad l;
  l.N = L->N;
  l.V1 = L->V1;
  l.V2 = L->V2;
  l.T = L->T;
  l.M1 = L->M1;
  l.M2 = L->M2;
  FailMode m = FailMode::None;
  const f64 ph = bond_utilization(P.bonds[0], l, fragility, table, &m);
  if (mode) *mode = static_cast<uint8_t>(m);
  return ph;
}

// K of the reference's build_matrix (core/src/stress/stress.cpp:84-132): call with null arrays
// for the sizes, then with arrays of those sizes. dof: n; rowptr: nfree + 1; col: nnzb;
// val: 36 nnzb.
int svxr_matrix(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb, const svxg_material* mats,
                int32_t* nfree, int64_t* nnzb, int32_t* dof, int32_t* rowptr, int32_t* col, double* val, double* id_scale) {
  MaterialTable table;
  fill_materials(table, mats);
  StressProblem P;
  P.mats = &table;
  fill_problem(P, nodes, n, bonds, nb);
  StressOptions so;
  so.amg_min_nodes = 1 << 30;  // (block-Jacobi: K alone)
  if (!P.assemble(so)) return 0;
  *nfree = P.K_.n;
  *nnzb = P.K_.blocks();
  if (dof) std::memcpy(dof, P.dof_.data(), sizeof(int32_t) * P.dof_.size());
  if (rowptr) std::memcpy(rowptr, P.K_.rowptr.data(), sizeof(int32_t) * P.K_.rowptr.size());
  if (col) std::memcpy(col, P.K_.col.data(), sizeof(int32_t) * P.K_.col.size());
  if (val) std::memcpy(val, P.K_.val.data(), sizeof(double) * P.K_.val.size());
  if (id_scale) *id_scale = P.id_scale_;
  return 1;
}

// The multigrid hierarchy of K before its single-precision conversion: every level's A, D^-1,
// aggregates (parent), prolongation and lambda_max estimate, and the coarsest dense factor.
void* svxr_hier_build(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb, const svxg_material* mats,
                      const svxg_stress_options* o, int32_t* ok) {
  MaterialTable table;
  fill_materials(table, mats);
  StressProblem P;
  P.mats = &table;
  fill_problem(P, nodes, n, bonds, nb);
  StressOptions so = options(o);
  const i32 min_nodes = so.amg_min_nodes;
  so.amg_min_nodes = 1 << 30;
  *ok = 0;
  if (!P.assemble(so)) return nullptr;
  (void)min_nodes;
  std::vector<V3> pos(size_t(P.nfree_));
  for (size_t i = 0; i < P.nodes.size(); ++i)
    if (P.dof_[i] >= 0) pos[size_t(P.dof_[i])] = P.nodes[i].c;
  Hier* h = new Hier;
  Amg& a = h->amg;
  a.opt_ = so.amg;
  a.lv_.clear();
  a.chol_.clear();
  a.chol_n_ = 0;
  a.work_ = 0;
  a.build_work_ = 0;
  if (P.K_.n == 0) {
    *ok = 1;
    return h;
  }
  a.lv_.emplace_back();
  a.lv_[0].A = P.K_;
  a.lv_[0].pos = pos;
  if (!a.finalize(a.lv_[0])) {
    delete h;
    return nullptr;
  }
  while (static_cast<int>(a.lv_.size()) < a.opt_.max_levels && a.lv_.back().A.n > a.opt_.coarse_max) {
    const Bsr6& L = a.lv_.back().A;
    const bool dense = a.lv_.size() > 1 && L.blocks() > 80 * static_cast<i64>(L.n);
    if (dense && !a.opt_.coarsen_dense) break;
    if (!a.coarsen(a.lv_.size() - 1, !dense && a.opt_.smoothed)) break;
    if (dense) break;
  }
  a.factor_coarsest();
  for (auto& L : a.lv_) h->lmax.push_back(a.estimate_lmax(L));
  *ok = 1;
  return h;
}

int32_t svxr_hier_levels(void* hp) { return static_cast<Hier*>(hp)->amg.levels(); }

int32_t svxr_hier_chol_n(void* hp) { return static_cast<Hier*>(hp)->amg.chol_n_; }

void svxr_hier_chol(void* hp, double* out) {
  const Hier* h = static_cast<Hier*>(hp);
  std::memcpy(out, h->amg.chol_.data(), sizeof(double) * h->amg.chol_.size());
}

void svxr_hier_dims(void* hp, int32_t l, int32_t* n, int64_t* nnzb, int64_t* pnnz) {
  const auto& L = static_cast<Hier*>(hp)->amg.lv_[size_t(l)];
  *n = L.A.n;
  *nnzb = L.A.blocks();
  *pnnz = static_cast<int64_t>(L.Pcol.size());
}

void svxr_hier_get(void* hp, int32_t l, int32_t* rowptr, int32_t* col, double* val, double* dinv, int32_t* parent,
                   int32_t* prow, int32_t* pcol, double* pval, double* pos, double* lmax) {
  const Hier* h = static_cast<Hier*>(hp);
  const auto& L = h->amg.lv_[size_t(l)];
  if (rowptr) std::memcpy(rowptr, L.A.rowptr.data(), sizeof(int32_t) * L.A.rowptr.size());
  if (col) std::memcpy(col, L.A.col.data(), sizeof(int32_t) * L.A.col.size());
  if (val) std::memcpy(val, L.A.val.data(), sizeof(double) * L.A.val.size());
  if (dinv) std::memcpy(dinv, L.Dinv.data(), sizeof(double) * L.Dinv.size());
  if (parent) std::memcpy(parent, L.parent.data(), sizeof(int32_t) * L.parent.size());
  if (prow) std::memcpy(prow, L.Prow.data(), sizeof(int32_t) * L.Prow.size());
  if (pcol) std::memcpy(pcol, L.Pcol.data(), sizeof(int32_t) * L.Pcol.size());
  if (pval) std::memcpy(pval, L.Pval.data(), sizeof(double) * L.Pval.size());
  if (pos)
    for (size_t i = 0; i < L.pos.size(); ++i) {
      pos[3 * i] = L.pos[i].x;
      pos[3 * i + 1] = L.pos[i].y;
      pos[3 * i + 2] = L.pos[i].z;
    }
  if (lmax) *lmax = h->lmax[size_t(l)];
}

void svxr_hier_free(void* hp) { delete static_cast<Hier*>(hp); }


// ---- section geometry: the world's own SecAcc::finish_lattice and section_strengths
// (core/src/world/world_internal.hpp:133-232, :370-399) on the given interfaces, bond k from
// secs[k], as World::Impl builds its bonds (core/src/world/world.cpp:839-850)

static svxg_v3 to3(const V3& v) { return svxg_v3{v.x, v.y, v.z}; }

void svxr_build_bonds(const svxg_node* nodes, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                      const svxg_junction* juncs, const svxg_lattice* lats, int32_t nl, int32_t samples,
                      const svxg_material* mats, svxg_bond* out) {
  MaterialTable table;
  fill_materials(table, mats);
  std::vector<LatticeXf> xfs(size_t(std::max(nl, 1)));
  for (int32_t g = 0; g < nl; ++g) {
    LatticeXf& X = xfs[size_t(g)];
    X.off = V3{lats[g].off[0], lats[g].off[1], lats[g].off[2]};
    for (int q = 0; q < 9; ++q) X.R.m[size_t(q)] = lats[g].R[q];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) X.Rt.m[size_t(3 * r + c)] = lats[g].R[3 * c + r];
    X.identity = lats[g].identity != 0;
  }
  for (int32_t k = 0; k < nb; ++k) {
    const svxg_section& S = secs[k];
    world_detail::SecAcc A;
    A.a = S.a;
    A.b = S.b;
    A.axis = S.axis;
    A.sign = S.sign;
    A.mb = static_cast<MaterialId>(S.mb);
    A.grid = S.grid;
    A.strength_b = S.strength_b;
    // (the voxels either side of each face and sample, by lattice)
    std::map<std::pair<uint16_t, IVec3>, world_detail::VoxelAt> vox;
    for (int32_t f = 0; f < S.faces; ++f) {
      const svxg_face& F = faces[S.first_face + f];
      IVec3 q{F.x, F.y, F.z};
      A.faces.push_back(q);
      A.fax.push_back(F.axis);
      A.fsg.push_back(F.sign);
      vox[{S.grid, q}] = world_detail::VoxelAt{F.vox_lo, F.damage_lo};
      q[F.axis] += 1;
      vox[{S.grid, q}] = world_detail::VoxelAt{F.vox_hi, F.damage_hi};
    }
    for (int32_t j = 0; j < S.junctions; ++j) {
      const svxg_junction& J = juncs[S.first_junction + j];
      world_detail::JSample js;
      js.v = IVec3{J.v[0], J.v[1], J.v[2]};
      js.o = IVec3{J.o[0], J.o[1], J.o[2]};
      js.vg = J.vg;
      js.og = J.og;
      js.face = J.face;
      js.sub = J.sub;
      js.kind = J.kind;
      A.js.push_back(js);
      A.jsg.push_back(J.sign);
      A.jw.push_back(J.weight);
      vox[{J.vg, js.v}] = world_detail::VoxelAt{J.vox_v, J.damage_v};
      if (J.kind != world_detail::kJunctionUnknown) vox[{J.og, js.o}] = world_detail::VoxelAt{J.vox_o, J.damage_o};
    }
    const V3 ca = v3(nodes[S.a].c);
    V3 cbv{};
    if (S.b >= 0) cbv = v3(nodes[S.b].c);
    const LatticeXf ident{};
    auto hx = [&](int g) { return nl > 0 ? lats[g].h : S.h; };
    auto xf = [&](int g) -> const LatticeXf& { return nl > 0 ? xfs[size_t(g)] : ident; };
    SBond B = A.finish(hx, xf, samples, ca, S.b >= 0 ? &cbv : nullptr, static_cast<MaterialId>(S.ma), S.strength_a);
    if (S.sectioned) {
      if (A.js.empty())
        world_detail::section_strengths(table, A.faces.data(), A.fax.data(), A.faces.size(),
                                        [&](const IVec3& p) { return vox[{S.grid, p}]; }, B);
      else
        world_detail::section_strengths_general(
            table, S.grid, A.faces.data(), A.fax.data(), A.faces.size(), A.js.data(), A.js.size(),
            [&](uint16_t g, const IVec3& p) { return vox[{g, p}]; }, B, samples);
    }
    svxg_bond& o = out[k];
    std::memset(&o, 0, sizeof(o));
    o.a = B.a;
    o.b = B.b;
    o.broken = B.broken ? 1 : 0;
    o.in_k = B.in_k ? 1 : 0;
    o.ma = static_cast<uint8_t>(B.ma);
    o.mb = static_cast<uint8_t>(B.mb);
    o.sectioned = B.sectioned ? 1 : 0;
    o.n = to3(B.n);
    o.t1 = to3(B.t1);
    o.t2 = to3(B.t2);
    o.area = B.area;
    o.p = to3(B.p);
    o.s1 = B.s1;
    o.s2 = B.s2;
    o.c1 = B.c1;
    o.c2 = B.c2;
    o.rmax = B.rmax;
    o.la = B.la;
    o.lb = B.lb;
    o.strength = B.strength;
    o.ft = B.ft;
    o.fb = B.fb;
    o.fc = B.fc;
    o.coh = B.coh;
    o.mu = B.mu;
    o.faces = B.faces;
    o.tag = k;
  }
}

// ---- one problem kept between calls (the judge's break rounds drive it: remove_bond,
// retire_nodes and solve on the same K, as World::Impl::judge does, core/src/world/world.cpp:1162-1277)

struct RefProblem {
  MaterialTable table;
  StressProblem P;
};

void* svxr_p_create(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb, const svxg_material* mats) {
  RefProblem* h = new RefProblem;
  fill_materials(h->table, mats);
  h->P.mats = &h->table;
  fill_problem(h->P, nodes, n, bonds, nb);
  return h;
}

void svxr_p_destroy(void* h) { delete static_cast<RefProblem*>(h); }

int svxr_p_assemble(void* h, const svxg_stress_options* o) { return static_cast<RefProblem*>(h)->P.assemble(options(o)) ? 1 : 0; }
int svxr_p_assembled(void* h) { return static_cast<RefProblem*>(h)->P.assembled() ? 1 : 0; }
void svxr_p_invalidate(void* h) { static_cast<RefProblem*>(h)->P.invalidate(); }
int svxr_p_preconditioner_current(void* h) { return static_cast<RefProblem*>(h)->P.preconditioner_current() ? 1 : 0; }
int svxr_p_block_jacobi(void* h) { return static_cast<RefProblem*>(h)->P.block_jacobi() ? 1 : 0; }

void svxr_p_solve(void* h, const double* f, double* u, double rtol, int32_t maxit, int32_t warm, svxg_pcg_result* res) {
  StressProblem& P = static_cast<RefProblem*>(h)->P;
  const size_t m = 6 * P.nodes.size();
  std::vector<f64> fv(f, f + m), uv(u, u + m);
  const PcgResult r = P.solve(fv, uv, rtol, maxit, warm != 0);
  std::memcpy(u, uv.data(), sizeof(double) * m);
  res->iters = r.iters;
  res->converged = r.converged;
  res->breakdown = r.breakdown;
  res->rel_res = r.rel_res;
}

void svxr_p_remove_bond(void* h, int32_t b) { static_cast<RefProblem*>(h)->P.remove_bond(b); }
void svxr_p_set_broken(void* h, int32_t b, int v) { static_cast<RefProblem*>(h)->P.bonds[size_t(b)].broken = v != 0; }

void svxr_p_retire_nodes(void* h, const int32_t* list, int32_t count) {
  static_cast<RefProblem*>(h)->P.retire_nodes(std::vector<i32>(list, list + count));
}

void svxr_p_bond_flags(void* h, uint8_t* broken, uint8_t* in_k) {
  const StressProblem& P = static_cast<RefProblem*>(h)->P;
  for (size_t k = 0; k < P.bonds.size(); ++k) {
    if (broken) broken[k] = P.bonds[k].broken ? 1 : 0;
    if (in_k) in_k[k] = P.bonds[k].in_k ? 1 : 0;
  }
}

void svxr_p_judge(void* h, const double* u, double fragility, svxg_bond_load* loads, double* phi, uint8_t* mode) {
  RefProblem* R = static_cast<RefProblem*>(h);
  const StressProblem& P = R->P;
  std::vector<f64> uv(u, u + 6 * P.nodes.size());
  for (size_t k = 0; k < P.bonds.size(); ++k) {
    const BondLoad L = P.bond_load(static_cast<i32>(k), uv);
    FailMode m = FailMode::None;
    const f64 ph = bond_utilization(P.bonds[k], L, fragility, R->table, &m);
    if (loads) loads[k] = svxg_bond_load{L.N, L.V1, L.V2, L.T, L.M1, L.M2};
    if (phi) phi[k] = ph;
    if (mode) mode[k] = static_cast<uint8_t>(m);
  }
}

// bond_utilization of every bond of the problem under the given loads (one per bond)
void svxr_p_utilization_many(void* h, const svxg_bond_load* loads, double fragility, double* phi, uint8_t* mode) {
  RefProblem* R = static_cast<RefProblem*>(h);
  const StressProblem& P = R->P;
  for (size_t k = 0; k < P.bonds.size(); ++k) {
    BondLoad l;
    l.N = loads[k].N;
    l.V1 = loads[k].V1;
    l.V2 = loads[k].V2;
    l.T = loads[k].T;
    l.M1 = loads[k].M1;
    l.M2 = loads[k].M2;
    FailMode m = FailMode::None;
    phi[k] = bond_utilization(P.bonds[k], l, fragility, R->table, &m);
    if (mode) mode[k] = static_cast<uint8_t>(m);
  }
}

void svxr_p_matrix(void* h, int32_t* nfree, int64_t* nnzb, int32_t* rowptr, int32_t* col, double* val) {
  const StressProblem& P = static_cast<RefProblem*>(h)->P;
  *nfree = P.K_.n;
  *nnzb = static_cast<int64_t>(P.K_.col.size());
  if (rowptr) std::memcpy(rowptr, P.K_.rowptr.data(), sizeof(int32_t) * P.K_.rowptr.size());
  if (col) std::memcpy(col, P.K_.col.data(), sizeof(int32_t) * P.K_.col.size());
  if (val) std::memcpy(val, P.K_.val.data(), sizeof(double) * P.K_.val.size());
}

// A loose piece's loads with the reference's own vector types, operators and
// StressProblem::add_force, in the lines of World::Impl::body_stress_run
// (core/src/world/world_pieces.cpp:566-603); the node of each force is given (the world maps a
// fragment through BodyGraph::frag_node).
void svxr_body_loads(const svxg_body_state* bs, const svxg_node* nodes, int32_t n, const svxg_v3* node_com,
                     const double* node_mass, const double* node_inertia, const svxg_point_force* forces,
                     int32_t nforces, int32_t inertia, double* out) {
  Body b;
  b.x = v3(bs->x);
  b.q = Quat{bs->q[0], bs->q[1], bs->q[2], bs->q[3]};
  b.com = v3(bs->com);
  b.w = v3(bs->w);
  for (int k = 0; k < 9; ++k) {
    b.inertia.m[size_t(k)] = bs->inertia[k];
    b.inv_inertia.m[size_t(k)] = bs->inv_inertia[k];
  }
  b.inv_mass = bs->inv_mass;
  const M3 R = to_matrix(b.q), Rt = transpose(R);
  std::vector<f64> f(6 * size_t(n), 0.0);
  const V3 g{0, 0, -bs->gravity};
  if (inertia) {
    V3 Ft, tau;
    for (int32_t k = 0; k < nforces; ++k) {
      Ft += v3(forces[k].F);
      tau += cross(v3(forces[k].p) - b.x, v3(forces[k].F));
    }
    const M3 Iw = R * b.inertia * Rt;
    const M3 Iwi = R * b.inv_inertia * Rt;
    const V3 a = Ft * b.inv_mass + g;
    const V3 alpha = Iwi * (tau - cross(b.w, Iw * b.w));
    for (int32_t i = 0; i < n; ++i) {
      M3 In;
      for (int k = 0; k < 9; ++k) In.m[size_t(k)] = node_inertia[9 * size_t(i) + size_t(k)];
      const V3 rw = R * (v3(node_com[i]) - b.com);
      const V3 ai = a + cross(alpha, rw) + cross(b.w, cross(b.w, rw));
      const V3 Fi = Rt * ((g - ai) * node_mass[i]);
      const M3 Ii = R * In * Rt;
      const V3 Mi = Rt * ((Ii * alpha + cross(b.w, Ii * b.w)) * -1.0);
      f64* fi = &f[6 * size_t(i)];
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
    StressProblem::add_force(f, i, v3(nodes[i].c), Rt * v3(forces[k].F), b.to_shape(v3(forces[k].p)));
  }
  std::memcpy(out, f.data(), sizeof(double) * f.size());
}

}  // extern "C"
