/* svxg.h - C ABI of the GB300 stress solve (hand-written sm_103a kernels, one GPU).
 *
 * This is the boundary a host binds in place of the reference's svx::StressProblem
 * (core/include/svx/stress/stress.hpp:74-160), the only solve type the reference's callers use
 * (World::Impl's Structure::P and BodyGraph::P, core/src/world/world_internal.hpp:745, :768).
 * Each entry point names the member it replaces. A problem owns its device buffers and one
 * CUDA stream; distinct problems may be driven from distinct host threads at the same time.
 *
 * Conventions: functions return SVXG_OK (0) or a negative SVXG_ERR_* code and never abort;
 * svxg_last_error() gives the calling thread's last message. Vectors f and u hold 6 doubles
 * per node (translation, rotation) in node order, fixed nodes 0, as the reference's.
 */
#ifndef SVXG_H
#define SVXG_H

#include <stddef.h>
#include <stdint.h>

#include "svxg_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SVXG_OK 0
#define SVXG_ERR_ARG (-1)      /* bad argument or size */
#define SVXG_ERR_CUDA (-2)     /* a CUDA call failed (message in svxg_last_error) */
#define SVXG_ERR_NOMEM (-3)    /* device memory (or the problem's budget) exhausted */
#define SVXG_ERR_STATE (-4)    /* not assembled / no graph */
#define SVXG_ERR_TIMEOUT (-5)  /* a bounded device wait gave up */
#define SVXG_ERR_NODEVICE (-6) /* no CUDA device */

typedef struct svxg_problem svxg_problem;

/* The reference's counters (Amg::level_sizes / level_blocks / work_per_apply / build_work,
 * amg.hpp:77-81; StressProblem::matrix_blocks / work_per_iteration / assembly_work,
 * stress.hpp:103-119) plus device bytes. */
typedef struct svxg_info {
  int32_t nfree, levels, block_jacobi, chol_n;
  int32_t level_sizes[16];
  int64_t level_blocks[32]; /* matrix blocks per level, then prolongation blocks per level */
  int64_t matrix_blocks, work_per_iteration, assembly_work, work_per_apply, build_work;
  int64_t device_bytes;     /* what the problem holds on the device now */
  int32_t precision;        /* SVXG_PRECISION_* of the last assemble */
  int32_t mixed_fallbacks;  /* mixed-precision solves since then finished in FP64 (FP32 stalled) */
  int64_t graph_bytes;      /* of device_bytes: the graph's copy (nodes, bonds, materials); the rest
                               is what svxg_release frees (StressProblem::solver_bytes) */
  double error_estimate;    /* the last solve's error against the FP64 solution, estimated as
                               ||M^-1 r|| / ||u|| from its final FP64 residual (solves under the
                               mixed-precision policy; 0 for FP64 ones) */
} svxg_info;

const char* svxg_last_error(void);
int svxg_device_count(void);

/* --- lifecycle (StressProblem's constructor / destructor) ----------------------------------- */
int svxg_problem_create(svxg_problem** out, int device);
void svxg_problem_destroy(svxg_problem* p);
/* The problem's CUDA stream (a cudaStream_t), for callers that order their own work on it. */
void* svxg_problem_stream(svxg_problem* p);

/* The graph: replaces the public members nodes, bonds, mats (stress.hpp:76-79). Copies them to
 * the device; the caller keeps its arrays. mats: SVXG_MAX_MATERIALS resolved entries. Call
 * again whenever the caller changed nodes or bonds between calls (invalidates the assembly). */
int svxg_set_graph(svxg_problem* p, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                   const svxg_material* mats);

/* The same from device memory of the problem's device (the graph kept on the GPU by the caller,
 * e.g. bonds made by svxg_build_bonds_device): copied device to device, with the host copies of
 * the nodes, each bond's nodes and flags and the materials read back; a bond with a node or
 * material out of range: SVXG_ERR_ARG and no graph. */
int svxg_set_graph_device(svxg_problem* p, const svxg_node* nodes_dev, int32_t n, const svxg_bond* bonds_dev,
                          int32_t nb, const svxg_material* mats_dev);

/* No counterpart in the reference (whose callers solve independent graphs one StressProblem each,
 * concurrently on pool threads, core/src/world/world_pieces.cpp:1460-1463). A batch: `count`
 * independent graphs as one problem, graph g's nodes and bonds after those of the graphs before it
 * (its bonds' node indices moved by its node offset), one material table. Assembly and the
 * multigrid are the reference's over that one graph (disjoint parts couple nowhere in K) with one
 * difference: aggregation keeps uncoupled leftover rows single instead of grouping them eight at a
 * time, so that the multigrid couples no two graphs either. Every launch covers the whole batch,
 * and the solve (svxg_solve / svxg_solve_device with f and u the graphs' vectors one after another)
 * runs one conjugate-gradient sequence per graph - its own alpha, beta, breakdown and stopping test
 * ||r_g|| <= rtol ||f_g|| - inside the shared launches, until every graph has stopped. The batch
 * lasts until the next svxg_set_graph / _device / reassemble. */
int svxg_set_graphs(svxg_problem* p, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                    const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats);
/* The same batch from graphs in device memory (pointer arrays on the host). */
int svxg_set_graphs_device(svxg_problem* p, int32_t count, const svxg_node* const* nodes_dev, const int32_t* n,
                           const svxg_bond* const* bonds_dev, const int32_t* nb, const svxg_material* mats_dev);
/* After a batch's solve: per graph ||r_g|| / ||f_g|| (0 without load), whether it met its target,
 * the iterations its sequence ran and, under the mixed-precision policy, its error estimate
 * (svxg_info.error_estimate; 0 otherwise). count: the batch's graph count; any array may be null. */
int svxg_graph_results(svxg_problem* p, int32_t count, double* rel_res, int32_t* converged, int32_t* iters,
                       double* err_est);

/* StressProblem::assemble (stress.hpp:83, stress.cpp:134-176): K over the intact bonds and the
 * preconditioner. *ok = 1 assembled, 0 singular diagonal (the reference's false). */
int svxg_assemble(svxg_problem* p, const svxg_stress_options* opt, int32_t* ok);
/* StressProblem::assembled / invalidate / preconditioner_current / block_jacobi (stress.hpp:84-92) */
int svxg_assembled(const svxg_problem* p);
int svxg_invalidate(svxg_problem* p);
int svxg_preconditioner_current(const svxg_problem* p);
int svxg_block_jacobi(const svxg_problem* p);
/* StressProblem::release (stress.hpp:99, stress.cpp:326-339): frees K, the hierarchy and the
 * run state; the graph stays. */
int svxg_release(svxg_problem* p);

/* StressProblem::reassemble (stress.hpp:110, stress.cpp:178-211) after the caller changed the
 * public members: the graph given here replaces the problem's, K is built again, the multigrid of
 * the last assemble keeps preconditioning the nodes it covered, and nodes appended since (free
 * indices from there on) get their own multigrid over K's appended block (24 nodes or more, when
 * it builds) or their block-Jacobi inverses, applied additively. Falls back to assemble when
 * nothing was assembled, the problem is block-Jacobi or free nodes were removed. *ok as assemble. */
int svxg_reassemble(svxg_problem* p, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                    const svxg_material* mats, int32_t* ok);
/* StressProblem::appended (stress.hpp:114): free nodes the multigrid does not cover. */
int32_t svxg_appended(const svxg_problem* p);
/* StressProblem::extend_warm_start (stress.hpp:113, stress.cpp:213-244): u (host, 6 n doubles,
 * in and out) with nodes first_new.. set from their intact bonds' older neighbours' rigid motion,
 * averaged over up to four passes, on the device. */
int svxg_extend_warm_start(svxg_problem* p, double* u, int32_t first_new);

/* StressProblem::remove_bond / retire_nodes (stress.hpp:108-109, stress.cpp:260-310): in-place
 * K downdates that keep the preconditioner. */
int svxg_remove_bond(svxg_problem* p, int32_t b);
int svxg_retire_nodes(svxg_problem* p, const int32_t* list, int32_t count);
/* remove_bond of each listed bond, in list order (the reference's loop of calls, e.g. a judge
 * round's breaks, world.cpp:1258-1270), with one device pass and one wait: K's blocks get the
 * same subtractions in the same order. */
int svxg_remove_bonds(svxg_problem* p, const int32_t* list, int32_t count);
/* The bonds' in_k / broken flags as the problem keeps them (the reference writes them into the
 * caller's bonds). Either pointer may be null. */
int svxg_bond_flags(svxg_problem* p, uint8_t* broken, uint8_t* in_k);

/* --- the solve ------------------------------------------------------------------------------ */
/* StressProblem::solve (stress.hpp:122, stress.cpp:348-360). f, u: host arrays of 6 n doubles;
 * u is the warm start when warm != 0 and the solution on return. maxit < 0: no cap. */
int svxg_solve(svxg_problem* p, const double* f, double* u, double rtol, int32_t maxit, int32_t warm,
               svxg_pcg_result* res);
/* The same with f and u in device memory (node order, 6 per node). */
int svxg_solve_device(svxg_problem* p, const double* f_dev, double* u_dev, double rtol, int32_t maxit, int32_t warm,
                      svxg_pcg_result* res);
/* StressProblem::begin / iterate / running / stop / current (stress.hpp:126-130, stress.cpp:362-475).
 * u0 may be null (cold start). */
int svxg_begin(svxg_problem* p, const double* f, const double* u0);
int svxg_iterate(svxg_problem* p, int32_t maxit, double rtol, svxg_pcg_result* res);
int svxg_running(const svxg_problem* p);
int svxg_stop(svxg_problem* p);
int svxg_current(svxg_problem* p, double* u);

/* --- bond loads and failure checks ------------------------------------------------------------ */
/* StressProblem::bond_load (stress.hpp:132, stress.cpp:477-502) of every bond, at u (host, 6 n)
 * or, when u is null, at the current solution. out: nb records. */
int svxg_bond_loads(svxg_problem* p, const double* u, svxg_bond_load* out);
/* bond_utilization (stress.hpp:64-66, stress.cpp:23-57) of every bond at the current solution:
 * phi (nb doubles) and mode (nb bytes, SVXG_FAIL_*), either may be null; over receives the
 * indices of the bonds with phi >= 1 in ascending order (capacity `cap`), *n_over their count. */
int svxg_utilization(svxg_problem* p, double fragility, double* phi, uint8_t* mode, int32_t* over, int32_t cap,
                     int32_t* n_over);

/* The same at the current solution with device outputs (phi: nb doubles, mode: nb bytes, over:
 * nb int32 - any may be null); *n_over (host) receives the failure count. */
int svxg_utilization_device(svxg_problem* p, double fragility, double* phi_dev, uint8_t* mode_dev, int32_t* over_dev,
                            int32_t* n_over);

/* No counterpart in the reference. The same judge for hosts that cannot let a library allocate
 * device memory (an engine that owns all of HBM through its own pool, whose frame loop must not
 * block on cudaMalloc/cudaFree): no problem handle, everything in the caller's device buffers -
 * the graph (nodes: n, bonds: nb, mats: SVXG_MAX_MATERIALS records), u (6 n doubles, node order),
 * phi (nb doubles), mode (nb bytes), over (nb int32; phi, mode and over may be null), on `stream`
 * (a cudaStream_t, null: the legacy default stream) of the current device; *n_over (host) gets
 * the failure count after the stream synchronizes. Allocates nothing: its scratch is one
 * 512 KiB array in the library's device image, so at most 16,777,216 bonds (more: SVXG_ERR_ARG).
 * A device's first call looks that array up (cudaGetSymbolAddress) and keeps its address for the
 * life of the process; do not call this after a cudaDeviceReset of that device. Each call
 * synchronizes `stream` before it returns (it reads the count back), so no call can run inside a
 * stream capture. Calls share the array: calls that overlap on the GPU race and must be ordered by
 * the caller. Node indices and material ids out of range: SVXG_ERR_ARG, those bonds skipped. */
int svxg_utilization_noalloc(const svxg_node* nodes_dev, int32_t n, const svxg_bond* bonds_dev, int32_t nb,
                             const svxg_material* mats_dev, const double* u_dev, double fragility, double* phi_dev,
                             uint8_t* mode_dev, int32_t* over_dev, int32_t* n_over, void* stream);

/* bond_strength / bond_utilization (stress.hpp:53-66, stress.cpp:14-57), the reference's free
 * functions, on the host from the same source as the device judge: out = ft, fb, fc, cohesion,
 * friction of the bond at `fragility`; utilization returns phi (-1 for a bad material id) and the
 * governing mode (SVXG_FAIL_*) in *mode (may be null). */
int svxg_bond_strength(const svxg_bond* b, double fragility, const svxg_material* mats, double* out);
double svxg_bond_utilization(const svxg_bond* b, const svxg_bond_load* L, double fragility, const svxg_material* mats,
                             uint8_t* mode);

/* --- loads ------------------------------------------------------------------------------------ */
/* World::Impl::load_vector (core/src/world/world.cpp:966-974): f (6 n) = each node's weight down z
 * plus ext (6 n, the loads applied to the structure; may be null). Host arrays. */
int svxg_structure_loads(int32_t n, const double* weight, const double* ext, double* f);
/* pin_reference (core/src/world/world_pieces.cpp:313-326): every node's `fixed` cleared, then the
 * node nearest com (the first of equals) fixed; returns its index (-1: no nodes). */
int32_t svxg_pin_reference(svxg_node* nodes, int32_t n, svxg_v3 com);
/* A loose piece's load (World::Impl::body_stress_run, world_pieces.cpp:566-603): with `inertia`,
 * each node's inertial relief from the piece's acceleration under gravity and the point forces -
 * translation and rotation of its centre (node_com, shape frame), its mass and inertia (node_inertia,
 * 9 per node, body frame) - then every point force on its node through add_force, in the shape
 * frame. f: 6 n, written. Host arrays. */
int svxg_body_loads(const svxg_body_state* b, const svxg_node* nodes, int32_t n, const svxg_v3* node_com,
                    const double* node_mass, const double* node_inertia, const svxg_point_force* forces,
                    int32_t nforces, int32_t inertia, double* f);

/* --- bonds from voxel faces -------------------------------------------------------------------- */
/* Replaces SecAcc::finish (finish_lattice / finish_general) + section_strengths /
 * section_strengths_general (core/src/world/world_internal.hpp:130-441), the section geometry
 * World::Impl runs for every bond it makes (core/src/world/world.cpp:839-850): bond k of out from
 * secs[k], its faces and its junction samples - the interface normal and frame, the elements'
 * projected centroid, principal axes, area, s1/s2, c1/c2/rmax, the spring lengths la/lb, the
 * strength multiplier (min of the two sides') and, where sectioned, the section strengths from
 * the voxels and damage either side of each face and sample (materials: SVXG_MAX_MATERIALS
 * records). A section without samples on an identity lattice takes finish_lattice, any other
 * finish_general, as the reference's dispatch does. lats (nl, indexed by a section's grid and a
 * sample's vg) may be null with nl = 0 when no section has samples (every lattice the
 * identity); a section's h is its faces' lattice's voxel size; samples: junction samples per face
 * edge. Bit for bit the reference's. Host arrays (nodes: n, secs: nb, faces: nf, juncs: nj, out:
 * nb); anything out of range: SVXG_ERR_ARG before anything runs. */
int svxg_build_bonds(const svxg_node* nodes, int32_t n, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                     int64_t nf, const svxg_junction* juncs, int64_t nj, const svxg_lattice* lats, int32_t nl,
                     int32_t samples, const svxg_material* mats, svxg_bond* out);
/* The same over device arrays on `stream` (a cudaStream_t; null: the legacy default stream),
 * allocating nothing; a section with anything out of range becomes a broken empty bond and
 * counts in *n_bad_dev (device int32, may be null). */
int svxg_build_bonds_device(const svxg_node* nodes_dev, int32_t n, const svxg_section* secs_dev, int32_t nb,
                            const svxg_face* faces_dev, int64_t nf, const svxg_junction* juncs_dev, int64_t nj,
                            const svxg_lattice* lats_dev, int32_t nl, int32_t samples, const svxg_material* mats_dev,
                            svxg_bond* out_dev, int32_t* n_bad_dev, void* stream);

/* --- the judge's break rounds ---------------------------------------------------------------- */
/* Replaces World::Impl::judge's cascade of one structure (core/src/world/world.cpp:1162-1277)
 * with its solve restarts (world.cpp:1041-1110) and detach_unsupported (world.cpp:1371-1458), on
 * this problem: solve (warm from u, at most o->maxit iterations; unconverged solves restart as
 * the world restarts them), judge every intact bond under lerp(judged, L, dif) while a shock is
 * on, break the round's worst bonds (thr = max(1, band x max phi), at least the worst quarter,
 * at most max_breaks_per_round) with remove_bond, retire what no support holds (their loads and
 * motion become zero), and again, until no bond is over strength or max_rounds rounds broke
 * bonds. opt: assemble()'s options (null: the last ones; a restart on a rebuilt preconditioner
 * sets amg_min_nodes = 0 as the world does); o: null for the defaults.
 * f: the load (6 n, host; not changed), u: the warm start in and the last solution out (6 n).
 * judged / judged_has: the bonds' last steady loads and whether they have one (nb each, in and
 * out; both null: none). phi: the last judgement's utilizations (nb, broken bonds 0), or null.
 * broken: the bonds the rounds broke, in order (up to broken_cap); retired: the nodes retired, in
 * order (up to retired_cap); res: counts and the final status (SVXG_CASCADE_*). The problem's
 * bonds and nodes are left broken and retired as the reference's would be (svxg_bond_flags). */
int svxg_cascade(svxg_problem* p, const svxg_stress_options* opt, const svxg_cascade_options* o, const double* f,
                 double* u, svxg_bond_load* judged, uint8_t* judged_has, double* phi, int32_t* broken,
                 int32_t broken_cap, int32_t* retired, int32_t retired_cap, svxg_cascade_result* res);

/* Replaces World::Impl::body_stress_run's break rounds of a loose piece within one substep
 * (core/src/world/world_pieces.cpp:614-808), on this problem: f (6 n, in and out) is the piece's
 * load - its inertial relief and point forces, built by the caller (add_force) - and comes back
 * with the chips' loads moved onto the piece; u (6 n) the warm start in, the last solution out.
 * Each round solves (o->maxit iterations at o->rtol; after the first round a failed solve
 * rebuilds the preconditioner once, then the rounds stop with u = 0), judges every intact bond
 * whose node a is not retired, breaks the worst (phi >= max(1, band x max phi), at least
 * ceil(round_fraction x over), at most max_breaks_per_round), each crack paid from o->energy when
 * it is >= 0 at fracture_energy x (crush_energy if it crushes) x area x min(Gf) x strength, and
 * stops when the energy runs out, nothing broke or it was the last round; otherwise the piece
 * splits from its pinned node (the last node with `fixed`): a part heavier than chip_fraction x
 * the piece ends the rounds, lighter parts (chips) pass their net force and moment on to the
 * nodes they broke from and retire. gf: fracture energy per material (SVXG_MAX_MATERIALS; null:
 * the reference presets'). opt: assemble()'s options (null: the last ones; the piece is
 * assembled with rtol = o->rtol, amg_min_nodes = 0 as the world does). broken / modes: the bonds
 * broken, in order, and their failure modes (up to broken_cap); chips: the chip nodes retired. */
int svxg_piece_rounds(svxg_problem* p, const svxg_stress_options* opt, const svxg_piece_options* o, const double* gf,
                      double* f, double* u, int32_t* broken, uint8_t* modes, int32_t broken_cap, int32_t* chips,
                      int32_t chips_cap, svxg_piece_result* res);

/* --- counters ------------------------------------------------------------------------------- */
int svxg_get_info(svxg_problem* p, svxg_info* info);
/* Kernel launches made by this library since it was loaded (all problems, all threads). */
int64_t svxg_launch_count(void);
/* The part of svxg_launch_count run as nodes of the solver's loop graphs (one graph launch per
 * solve from the host; the rest were launched one by one from host threads). */
int64_t svxg_graph_launch_count(void);
/* Live timing of the conjugate-gradient SpMV: CUDA events on the problem's stream around each of
 * its launches while enabled; read returns their summed duration (ms) and count, and resets. */
int svxg_timer_enable(svxg_problem* p, int32_t on);
int svxg_timer_read(svxg_problem* p, double* ms_total, int64_t* launches);
/* The same for a chosen kernel: SVXG_TIMER_CG_SPMV (as svxg_timer_enable) or
 * SVXG_TIMER_GALERKIN_AP (the multigrid build's A P values kernel, every level of each assemble);
 * read_work also gives the timed launches' algorithmic units (Galerkin: 6x6 by 6x6 block products,
 * 432 FP64 operations each) and resets. */
enum { SVXG_TIMER_CG_SPMV = 0, SVXG_TIMER_GALERKIN_AP = 1 };
int svxg_timer_enable_kernel(svxg_problem* p, int32_t kind, int32_t on);
int svxg_timer_read_work(svxg_problem* p, double* ms_total, int64_t* launches, int64_t* work);
/* The conjugate-gradient SpMV timed alone: `reps` back-to-back launches of the kernel an iteration
 * runs on the assembled K (q = K p with p.q fused; precision SVXG_PRECISION_FP64: the FP64 K,
 * otherwise the mixed sequence's FP32 K), each doing its work, CUDA events on the problem's
 * stream; *ms_per_launch their mean. The problem's run state is not touched. */
int svxg_time_spmv(svxg_problem* p, int32_t precision, int32_t reps, double* ms_per_launch);
/* This GPU's FP64 fused multiply-add throughput (TFLOP/s, 2 per FMA), measured by independent FMA
 * chains over every SM: the ceiling of the FP64-issue-bound kernels. */
int svxg_measure_fp64_rate(int device, double* tflops);

/* --- parity access (tests) ------------------------------------------------------------------ */
/* K as assembled: call with null arrays for *nfree / *nnzb, then with arrays of those sizes. */
int svxg_debug_matrix(svxg_problem* p, int32_t* nfree, int64_t* nnzb, int32_t* dof, int32_t* rowptr, int32_t* col,
                      double* val, double* id_scale);
/* One multigrid level in double precision: sizes, then arrays (any may be null). */
int svxg_debug_level_dims(svxg_problem* p, int32_t level, int32_t* n, int64_t* nnzb, int64_t* pnnz);
int svxg_debug_level(svxg_problem* p, int32_t level, int32_t* rowptr, int32_t* col, double* val, double* dinv,
                     int32_t* parent, int32_t* prow, int32_t* pcol, double* pval, double* pos, double* lmax);
/* z = M^-1 r and y = K x over the free DOFs (host arrays of 6 nfree). */
int svxg_debug_precondition(svxg_problem* p, const double* r, double* z);
/* sqrt of ((0 + v0^2) + v1^2) + ... summed in index order, computed in parallel on the device
 * (the multigrid setup's exact norm): for checking it against a sequential host loop. */
int svxg_debug_seq_norm(const double* v, int64_t n, double* out);
int svxg_debug_apply(svxg_problem* p, const double* x, double* y);

/* Schedule timings of the last assemble, recorded when the environment sets SVXG_TUNE_LOG=1 or
 * SVXG_TUNE_LIVE=1 before the library loads (the autotuner's input): per BSR operator its kind
 * (0: K in FP64, 1: a level's A in FP32, 2: prolongation, 3: restriction), level, block rows,
 * blocks and the time of three products with each row schedule. Without them the schedules come
 * from the committed table alone and nothing is timed. */
typedef struct svxg_tune_entry {
  int32_t kind, level;
  int64_t rows, blocks;
  float ms_warp_row, ms_group_row;
} svxg_tune_entry;
int svxg_debug_tune_log(svxg_problem* p, svxg_tune_entry* out, int32_t cap, int32_t* count);

/* Per-phase device times of the calls made while on (an event recorded on the problem's stream at
 * each phase boundary of assemble - K, then per level aggregation, positions, lambda_max,
 * prolongation, restriction lists, A P, coarse pattern, coarse values, the level's end - the
 * coarsest factor, and of a host solve; no host wait). svxg_phase_times waits for the stream and
 * gives, from the last assemble (or reassemble) on, each phase's label and milliseconds since the
 * previous boundary; *count = the phases recorded (out holds at most cap). */
typedef struct svxg_phase_time {
  char label[48];
  double ms;
} svxg_phase_time;
int svxg_phase_timing(svxg_problem* p, int32_t on);
int svxg_phase_times(svxg_problem* p, svxg_phase_time* out, int32_t cap, int32_t* count);

/* The host-side trace of the last assemble and host solve when the environment sets SVXG_TRACE=1
 * before the library loads (the stream is drained at each mark, so device time lands on the
 * phase that queued it): lines of "microseconds since the assemble began, since the previous
 * mark, label". Returns the text's length; writes at most cap - 1 characters and a 0. */
int svxg_debug_trace(svxg_problem* p, char* out, int32_t cap);

#ifdef __cplusplus
}
#endif

#endif /* SVXG_H */
