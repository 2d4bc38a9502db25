/* svx_oracle.h - TEST INFRASTRUCTURE ONLY: the oracle (a CPU restatement of the reference's stress
 * solve in plain C). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
 * as the checker or as the timed CPU baseline; the shipped library never does.
 *
 * It restates, operation for operation (same summation orders, no fused multiply-adds: built with
 * -ffp-contract=off), the reference's
 *   core/src/stress/stress.cpp  (StressProblem: build_matrix, assemble, begin/iterate/solve,
 *                                bond_load, bond_strength, bond_utilization, remove_bond,
 *                                retire_nodes)
 *   core/src/solve/amg.cpp      (Bsr6, Bsr6Builder, Amg: finalize, estimate_lmax, build,
 *                                coarsen, factor_coarsest, make_fast, smooth_f, cycle_f, apply;
 *                                blk6::inv6, fro6, rigid_block, atbd_add)
 * so that its results are bit-identical to the reference's on any input (pinned by
 * tests/test_oracle_pin.py against the reference compiled from source, and by the golden
 * fixtures under tests/golden/). Row-parallel loops use OpenMP over the reference's fixed
 * chunks (512 rows, dots in 4096-element chunks), so results do not depend on the thread count.
 */
#ifndef SVX_ORACLE_H
#define SVX_ORACLE_H

#include <stdint.h>

#include "svxg_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct svxo_problem svxo_problem;

typedef struct svxo_info {
  int32_t nfree, levels, block_jacobi, chol_n;
  int32_t level_sizes[16];
  int64_t level_blocks[32];
  int64_t matrix_blocks, work_per_iteration, assembly_work, work_per_apply, build_work;
} svxo_info;

void svxo_set_threads(int n);
/* pass 3 groups uncoupled leftover rows eight at a time (1, the reference) or keeps each single (0,
   the library's batches of graphs) */
void svxo_set_group_isolated(int on);
int svxo_num_threads(void);

svxo_problem* svxo_create(const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                          const svxg_material* mats);
void svxo_destroy(svxo_problem* P);
/* StressProblem::assemble (stress.cpp:134-176). 1: assembled, 0: singular. */
int svxo_assemble(svxo_problem* P, const svxg_stress_options* opt);
/* StressProblem::solve (stress.cpp:348-360); u: 6 per node, in (warm) and out. */
int svxo_solve(svxo_problem* P, const double* f, double* u, double rtol, int32_t maxit, int32_t warm,
               svxg_pcg_result* res);
void svxo_begin(svxo_problem* P, const double* f, const double* u0 /* NULL: cold */);
int svxo_iterate(svxo_problem* P, int32_t maxit, double rtol, svxg_pcg_result* res);
void svxo_current(const svxo_problem* P, double* u);
void svxo_remove_bond(svxo_problem* P, int32_t b);
void svxo_retire_nodes(svxo_problem* P, const int32_t* list, int32_t count);
void svxo_get_info(const svxo_problem* P, svxo_info* info);
/* the bonds' in_k flags as the problem keeps them */
void svxo_bond_flags(const svxo_problem* P, uint8_t* broken, uint8_t* in_k);

/* bond_load / bond_utilization of every bond at u (6 per node). */
void svxo_judge(const svxo_problem* P, const double* u, double fragility, svxg_bond_load* loads, double* phi,
                uint8_t* mode);
double svxo_utilization(const svxg_bond* b, const svxg_bond_load* L, double fragility, const svxg_material* mats,
                        uint8_t* mode);

/* bond_utilization of every bond under the given loads (one per bond). */
void svxo_utilization_many(const svxo_problem* P, const svxg_bond_load* loads, double fragility, double* phi,
                           uint8_t* mode);
/* bonds[b].broken = v (a caller's write to the public member). */
void svxo_set_broken(svxo_problem* P, int32_t b, int v);
/* StressProblem::invalidate / assembled / preconditioner_current (stress.hpp:83-91). */
void svxo_invalidate(svxo_problem* P);
int svxo_assembled(const svxo_problem* P);
int svxo_preconditioner_current(const svxo_problem* P);

/* The bonds of the given interfaces: SecAcc::finish (finish_lattice / finish_general) +
 * section_strengths / section_strengths_general (core/src/world/world_internal.hpp:130-441),
 * bond k from secs[k]; lattices (by section grid and sample vg) and junctions may be NULL when
 * no section has junction samples and every faces' lattice is the identity; samples: junction
 * samples per face edge. */
void svxo_build_bonds(const svxg_node* nodes, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                      const svxg_junction* juncs, const svxg_lattice* lats, int32_t samples,
                      const svxg_material* mats, svxg_bond* out);

/* K (after svxo_assemble). rowptr: nfree + 1, col: nnzb, val: 36 nnzb, dof: n. */
void svxo_matrix_dims(const svxo_problem* P, int32_t* nfree, int64_t* nnzb);
void svxo_matrix(const svxo_problem* P, int32_t* dof, int32_t* rowptr, int32_t* col, double* val, double* id_scale);

/* The multigrid hierarchy kept in double precision (svxo_assemble with keep_levels set first).
 * Level l: A (rowptr/col/val), D^-1, aggregates (parent), prolongation (Prow/Pcol/Pval),
 * positions (3 per node), lambda_max estimate. */
void svxo_keep_levels(svxo_problem* P, int keep);
int32_t svxo_levels(const svxo_problem* P);
void svxo_level_dims(const svxo_problem* P, int32_t l, int32_t* n, int64_t* nnzb, int64_t* pnnz);
void svxo_level_get(const svxo_problem* P, int32_t l, int32_t* rowptr, int32_t* col, double* val, double* dinv,
                    int32_t* parent, int32_t* prow, int32_t* pcol, double* pval, double* pos, double* lmax);
int32_t svxo_chol_n(const svxo_problem* P);
void svxo_chol(const svxo_problem* P, double* out);
/* One application of the preconditioner (Amg::apply / block-Jacobi) to r (6 per free node). */
void svxo_precondition(const svxo_problem* P, const double* r, double* z);
/* y = K x over the free DOFs (Bsr6::apply). */
void svxo_apply_k(const svxo_problem* P, const double* x, double* y);

/* Exact sequential double sum of nonnegative terms, in index order (the reference's loops
 * `s += a[k]`): a helper for checking the device's exact summation. */
double svxo_seq_sum(const double* a, int64_t n);

/* Loads: World::Impl::load_vector (world.cpp:966-974), pin_reference (world_pieces.cpp:313-326),
 * body_stress_run's inertial relief and point forces (world_pieces.cpp:566-603). */
void svxo_structure_loads(int32_t n, const double* weight, const double* ext, double* f);
int32_t svxo_pin_reference(svxg_node* nodes, int32_t n, svxg_v3 com);
void svxo_body_loads(const svxg_body_state* b, const svxg_node* nodes, int32_t n, const svxg_v3* node_com,
                     const double* node_mass, const double* node_inertia, const svxg_point_force* forces,
                     int32_t nforces, int32_t inertia, double* f);

#ifdef __cplusplus
}
#endif

#endif /* SVX_ORACLE_H */
