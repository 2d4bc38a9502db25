// problem.cuh - device state of one stress problem and the launchers each translation unit owns.
//
// HBM layout of a problem (all device-resident between calls):
//   graph:  nodes (AoS svxg_node, 40 B), bonds (AoS svxg_bond, 216 B), material table (8 KB)
//   K:      BSR of 6x6 blocks: rowptr[nfree+1] i32, col[nnzb] i32, val[36 nnzb] f64 row-major,
//           each block row contiguous (a warp reads a row's blocks as one stream)
//   K32:    the same values in f32 (mixed precision)
//   hierarchy: per level A (BSR f64 for setup, f32 copy for the cycle), D^-1 (f64, f32),
//           prolongation (BSR by fine row) and restriction (by coarse row) in f32, vectors of
//           6 per node
//   run:    x, r, z, p, q (6 nfree f64), the load, scalars of the conjugate-gradient sequence
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "svxg.h"

namespace svxg {

// Thread-local last error message (svxg_last_error).
void set_error(const std::string& msg);

// Kernel launches made by this library (svxg_launch_count): every launch site counts itself.
void count_launch();
#define SVXG_COUNT_LAUNCH() ::svxg::count_launch()

#define SVXG_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      ::svxg::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));              \
      return SVXG_ERR_CUDA;                                                               \
    }                                                                                     \
  } while (0)

// Stream-ordered device allocation from the library's memory pool of the current device (one
// per device, created on first use): memory freed by a problem stays in the pool for the next
// problem, and neither allocation nor release synchronizes the device, so problems on other
// streams keep running while one is built or torn down.
cudaError_t pool_malloc_async(void** p, size_t bytes, cudaStream_t s);
// The calling thread's pool (current device) keeps at most `keep` unused bytes.
void pool_trim(size_t keep);

// Waits on the host until `s` has drained. Spins (cudaStreamSynchronize) by default; while
// blocking waits are on - a server with several slots holds them on, so that the slots' host
// threads sleep instead of competing for cores while their streams run - it sleeps on an event.
cudaError_t host_wait(cudaStream_t s);
void blocking_waits(bool on);  // counted: on/off pairs nest

// Device allocations of a problem (counted against its bytes), ordered on its stream.
struct DevArena {
  cudaStream_t stream = nullptr;
  std::vector<std::pair<void*, size_t>> live;
  int64_t bytes = 0;
  template <class T>
  int alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void* q = nullptr;
    cudaError_t e = pool_malloc_async(&q, count * sizeof(T), stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(std::string("device allocation: ") + cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? SVXG_ERR_NOMEM : SVXG_ERR_CUDA;
    }
    live.push_back({q, count * sizeof(T)});
    bytes += int64_t(count * sizeof(T));
    *p = static_cast<T*>(q);
    return SVXG_OK;
  }
  template <class T>
  void release(T*& p) {
    if (!p) return;
    for (size_t i = 0; i < live.size(); ++i)
      if (live[i].first == p) {
        cudaFreeAsync(p, stream);
        bytes -= int64_t(live[i].second);
        live[i] = live.back();
        live.pop_back();
        break;
      }
    p = nullptr;
  }
  // [p, p + bytes) inside one live allocation (a host-side guard before copies)
  bool holds(const void* p, size_t bytes) const {
    const char* c = static_cast<const char*>(p);
    for (const auto& e : live) {
      const char* b = static_cast<const char*>(e.first);
      if (c >= b && c + bytes <= b + e.second) return true;
    }
    return false;
  }
  void release_all() {
    for (auto& e : live) cudaFreeAsync(e.first, stream);
    live.clear();
    bytes = 0;
  }
};

struct Bsr {
  int32_t n = 0;
  int64_t nnzb = 0;
  int32_t* rowptr = nullptr;
  int32_t* col = nullptr;
  double* val = nullptr;  // 36 per block, row-major
  float* val32 = nullptr; // 36 per block, row-major (f32 copy)
};

// The scalars of a conjugate-gradient run (device memory).
struct PcgScalars {
  double rz, bn, target, pq, alpha, beta, rn, rel_res;
  int32_t iters, converged, breakdown, done;
  int32_t maxit, pad0;
  double rr, rz_new;
};

struct Level {
  Bsr A;
  double* dinv = nullptr;    // 36 per node (f64, setup)
  float* dinv32 = nullptr;   // 36 per node (f32, cycle)
  int32_t* parent = nullptr; // node -> coarse node
  double* pos = nullptr;     // 3 per node
  int32_t* prow = nullptr;   // prolongation by fine row
  int32_t* pcol = nullptr;
  double* pval = nullptr;
  float* pval32 = nullptr;
  int64_t pnnz = 0;
  int32_t* rrow = nullptr;   // restriction by coarse row: entries (fine node, P block)
  int32_t* rent_i = nullptr;
  int32_t* rent_e = nullptr;
  double lmax = 0.0;         // lambda_max(D^-1 A) estimate (smoothed prolongation's damping)
  double cheb_lmax = 0.0;    // the smoother's estimate
  float* b32 = nullptr;      // cycle vectors, 6 per node (f32)
  float* x32 = nullptr;
  float* r32 = nullptr;
  float* t32 = nullptr;
  float* u32 = nullptr;
  int sched_a = 0, sched_p = 0, sched_r = 0;  // row-product schedules (spmv_row.cuh), autotuned
  const int32_t* gmap = nullptr;  // a batch's: each row's graph (-1: unknown), in Problem::d_seg_lmap
};

struct Problem {
  int device = 0;
  cudaStream_t stream = nullptr;
  // stream and pinned mirrors (h_s, h_ms) lent by a server slot for the duration of a request,
  // not owned: destroy leaves them alone
  bool borrowed = false;
  DevArena mem;
  // graph (host copy kept for the in-place updates' bookkeeping)
  int32_t n = 0, nb = 0;
  std::vector<svxg_node> h_nodes;
  // per bond: its nodes (a, b) and its flags as the problem keeps them (the 216-byte records
  // themselves live on the device only: a host pass over them costs milliseconds on large graphs)
  std::vector<int32_t> h_bond_ab;
  std::vector<uint8_t> h_broken, h_in_k;
  std::vector<svxg_material> h_mats;
  svxg_node* d_nodes = nullptr;
  svxg_bond* d_bonds = nullptr;
  svxg_material* d_mats = nullptr;
  bool have_graph = false;
  // assembly
  svxg_stress_options opt{};
  bool assembled = false, pc_current = false, jacobi_only = false;
  int32_t pc_n = 0;               // free nodes the multigrid covers (nodes appended since: pc_n..nfree)
  Problem* sub = nullptr;         // the appended nodes' own multigrid (reassemble), owned
  int64_t assembly_work = 0;
  int32_t nfree = 0;
  int32_t* d_dof = nullptr;       // node -> free index (-1 fixed)
  std::vector<int32_t> h_dof;
  uint8_t* d_in_k = nullptr;      // per bond
  Bsr K;
  double id_scale = 1.0;
  double* d_jinv = nullptr;       // block-Jacobi inverses (36 per free node)
  int sched_k64 = 0, sched_k32 = 0;  // K's SpMV schedules (FP64 CG, FP32 inner), autotuned
  int4* d_kslots = nullptr;       // K's block rows by length as slots (the FP64 CG products' schedule), or null
  // a batch: several independent graphs as one problem (svxg_set_graphs), graph g its nodes
  // [seg_node[g], seg_node[g + 1]) and bonds [seg_bond[g], seg_bond[g + 1]); the solve stops when
  // every graph meets its own target (segmented norms over its free rows d_seg_row[g] ..)
  int32_t seg_n = 0;
  std::vector<int64_t> seg_node, seg_bond;
  int32_t* d_seg_row = nullptr;   // seg_n + 1 free-row offsets (made at assembly)
  int32_t* d_seg_of_row = nullptr;  // each free row's graph
  double* d_seg = nullptr;        // per graph: its sequence's scalars (solve.cu kSegF)
  int32_t* d_seg_flag = nullptr;  // per graph: 0 running, 1 converged, 2 broken down
  int32_t* d_seg_lmap = nullptr;  // every coarse level's row -> graph (Level::gmap; level 0: d_seg_of_row)
  // set while a batch's iteration body is enqueued: its kernels skip the rows of stopped graphs
  const int32_t* skip_flag = nullptr;
  // multigrid
  std::vector<Level> lv;
  double* d_chol = nullptr;       // coarsest dense factor (m x m, lower = L, upper = L^T)
  double* d_cinv = nullptr;       // its inverse L^-1 (lower), for the cycle's coarsest solve
  double* d_cvec = nullptr;       // coarsest solve's f64 vectors (2 m)
  int32_t chol_n = 0;
  int64_t amg_work = 0, amg_build_work = 0;
  // run state
  double *d_x = nullptr, *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_q = nullptr, *d_f = nullptr;
  double* d_un = nullptr;         // node-order u then f (12 n), owned by the C ABI's calls
  PcgScalars* d_s = nullptr;
  PcgScalars* h_s = nullptr;      // pinned mirror
  const int32_t* cycle_stop = nullptr;  // the running sequence's done flag: cycle kernels return at once when set
  float* d_mx = nullptr;          // mixed precision: d, r, z, p, q in f32 (5 x 6 nfree)
  void* d_ms = nullptr;           // mixed precision scalars (device)
  void* h_ms = nullptr;           // ... pinned mirror
  int32_t mx_maxit = 0;
  int32_t mixed_fallbacks = 0;    // mixed runs finished by the FP64 sequence (since assemble)
  double last_err_est = 0.0;      // the last mixed-policy solve's error estimate (solve.cu error_estimate)
  double* d_partials = nullptr;   // block partial sums
  unsigned* d_counter = nullptr;  // last-block counters
  int32_t partial_blocks = 0;
  bool active = false;
  int32_t run_iters = 0;
  int32_t host_loops = 0;         // host-driven iterate() runs since the last assemble
  void* d_bdesc = nullptr;        // block_solve.cu: the levels' descriptor of a small problem
  float* d_cinv32 = nullptr;      // ... and its coarsest inverse in f32
  // whole-iterate graphs (graphs.cu): built on first use after each assemble
  void* loop_plain = nullptr;
  void* loop_mixed = nullptr;
  // live kernel timing (CUDA events around each conjugate-gradient SpMV launch)
  bool timer_on = false;
  int32_t timer_kind = 0;         // SVXG_TIMER_*: the kernel timed
  std::vector<cudaEvent_t> timer_events;
  size_t timer_used = 0;          // event pairs recorded since the last read
  int64_t timer_work = 0;         // algorithmic units of the timed launches (SVXG_TIMER_GALERKIN_AP: block products)
  bool spmv_timer() const { return timer_on && timer_kind == SVXG_TIMER_CG_SPMV; }
  // per-phase device timing (svxg_phase_timing): an event on the stream at each trace mark, no
  // host wait; read back by svxg_phase_times
  bool phase_on = false;
  std::vector<cudaEvent_t> phase_events;
  std::vector<const char*> phase_labels;
  size_t phase_used = 0;
  // host-side trace of the last assemble and solve (SVXG_TRACE=1): label, microseconds since the
  // assemble began, with the stream drained at each mark so device time is attributed
  std::vector<std::pair<const char*, double>> trace;
  // row-schedule timings of the last assemble (kept only when the environment asks for them)
  std::vector<svxg_tune_entry> tune_log;
  // scratch
  int32_t* d_scan = nullptr;      // scan block sums
  int64_t scan_cap = 0;
  int32_t* d_rm_head = nullptr;   // exact_cascade.cu: a chain head per block of K (-1 between calls)
  int64_t rm_head_cap = 0;
};

// Marks a point of the host-side trace when SVXG_TRACE=1 (drains the problem's stream first);
// does nothing otherwise. `restart` begins a new trace.
void trace_mark(Problem& P, const char* label, bool restart = false);

// ---- launchers (one translation unit each) ---------------------------------------------------
// capi.cu
enum WarmStart { kCold = 0, kWarmHost = 1, kWarmResident = 2 };
// f, u (6 per node) host or device memory; kWarmResident starts from the problem's last solution,
// still on the device
int batch_solve_loads(Problem& P, const double* const* f, const uint8_t* take, double* const* u_out, double rtol,
                      int32_t maxit, bool warm, svxg_pcg_result* res);  // capi.cu: a batch's solve
int solve_nodes_host(Problem& P, const double* f, double* u, double rtol, int32_t maxit, int warm,
                     svxg_pcg_result* res);
int ensure_node_vectors(Problem& P);
// exact_assemble.cu
int assemble_matrix(Problem& P);                 // dof, pattern, K, id_scale, identity rows
int build_jacobi(Problem& P);                    // block-Jacobi inverses
int remove_bonds_device(Problem& P, const int32_t* bonds, int32_t count);  // sequential, in order
int set_identity_rows(Problem& P, const int32_t* rows, int32_t count);
// exact_amg.cu
int build_hierarchy(Problem& P, int32_t* ok);    // Amg::build on the device, bit for bit
int build_hierarchy_fast(Problem& P, int32_t* ok);  // the same with FMAs and a tree-summed norm
// the multigrid of the problem's arithmetic: bit for bit in FP64, the fast build under the
// mixed-precision policy (whose cycle and inner sequences run in FP32 anyway)
inline int build_multigrid(Problem& P, int32_t* ok) {
  return P.opt.precision == SVXG_PRECISION_FP64 ? build_hierarchy(P, ok) : build_hierarchy_fast(P, ok);
}
int debug_seq_norm(cudaStream_t st, const double* v, int64_t n, double* out_dev);
// dense.cu: C (m x m, the coarsest operator) -> chol (L, L^T mirrored above; may alias C) and
// cinv (L^-1, then L^-T), all device, m x m row-major
int dense_factor_inverse(Problem& P, int32_t m, const double* C, double* chol, double* cinv);
// solve.cu
int spmv(Problem& P, const Bsr& A, const double* x, double* y);
int pcg_begin(Problem& P, const double* f_nodes, const double* u0_nodes);  // device, node order
int pcg_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res);
int plain_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res);  // the FP64 sequence
int pcg_restart_fp64(Problem& P);                 // FP64 sequence restarted from the current x
int gather_solution(Problem& P, double* u_nodes);                        // device, node order
int precondition(Problem& P, const double* r, double* z);
int free_run(Problem& P);
int tune_k64(Problem& P);
int time_cg_spmv(Problem& P, int32_t reps, float* ms_per_launch);    // solve.cu
int seg_prepare(Problem& P);   // solve.cu: a batch's free-row offsets and per-graph scalars after assembly
int seg_results(Problem& P, double* rel_res, int32_t* converged, int32_t* iters, double* err_est);  // solve.cu
int error_estimate(Problem& P);  // solve.cu: ||M^-1 r|| / ||x|| after a solve (per graph in a batch)
int seg_launch(Problem& P, int op, const double* a, const double* b, double rtol);  // solve.cu
int time_cg_spmv32(Problem& P, int32_t reps, float* ms_per_launch);  // mixed.cu
int measure_fp64_rate(int device, double* tflops);                    // tune.cu
// tune.cu: the row schedule of a BSR operator (spmv_row.cuh), from the committed table (a pure
// function of the operator's shape, so results never depend on timing); the timings are taken
// and logged only when the environment asks (SVXG_TUNE_LOG=1; SVXG_TUNE_LIVE=1 also lets them
// decide)
enum OpKind { kOpK64 = 0, kOpA32 = 1, kOpP32 = 2, kOpR32 = 3 };
int table_sched(int kind, int64_t rows, int64_t blocks);
bool tune_timing();
int tune_decide(Problem& P, int kind, int level, int64_t rows, int64_t blocks, float ms_warp, float ms_group);
// block_solve.cu: a small problem's AMG iterate() in one block launch
constexpr int32_t kBlockSolveMax = 1536;
bool block_solve_fits(const Problem& P);
int block_iterate(Problem& P);
// exact_appended.cu (StressProblem::reassemble / extend_warm_start)
int build_appended(Problem& P);                  // P.sub over K's appended block (>= 24 nodes)
void release_appended(Problem& P);
int precondition_amg(Problem& P, const double* r, double* z);  // the multigrid, plus the appended part
int extend_warm_start_device(Problem& P, double* u_nodes, int32_t first_new);
// vcycle.cu
int vcycle(Problem& P, const double* r, double* z);
int vcycle32(Problem& P, const float* r, float* z);
// mixed.cu
int mixed_begin(Problem& P);
int mixed_iterate(Problem& P, int32_t maxit, double rtol, svxg_pcg_result* res);
int prepare_cycle(Problem& P);
// exact_judge.cu
int bond_loads_device(Problem& P, const double* u_nodes, svxg_bond_load* out);
int utilization_device(Problem& P, const double* u_nodes, double fragility, double* phi, uint8_t* mode,
                       int32_t* over, int32_t* n_over);
// graphs.cu
bool use_graphs();
bool seg_skip(const Problem& P);  // a batch's iteration bodies skip stopped graphs' rows
constexpr int32_t kGraphMinFree = 4096;
// K of at least this many block rows gets its rows sorted by length for the conjugate-gradient
// products (solve.cu build_row_slots): one host round trip of K's row pointers at assembly.
#ifndef SVXG_SORTED_MIN_ROWS
#define SVXG_SORTED_MIN_ROWS 4096
#endif
constexpr int32_t kSortedMinRows = SVXG_SORTED_MIN_ROWS;
// The FP32 inner sequences (FP32 K SpMV and Krylov vectors inside FP64 refinement) run under
// SVXG_PRECISION_MIXED_ALL only. On this part they never paid: the FP32 sequences need about twice
// the iterations, and the FP32 V-cycle, which the FP64 sequence runs too, dominates an iteration -
// so the mixed policy (SVXG_PRECISION_MIXED) runs the FP64 sequence with the FP32 V-cycle and the
// fast multigrid build at every size
inline bool mixed_run(const Problem& P) {
  // (a batch runs the FP64 sequence: its stopping test is per graph)
  if (P.jacobi_only || P.pc_n < P.nfree || !P.K.val32 || P.seg_n > 0) return false;
  return P.opt.precision == SVXG_PRECISION_MIXED_ALL;
}
bool loop_graph_worth(const Problem& P, const void* slot);
int timer_mark(Problem& P, bool closing = false);
int run_loop(Problem& P, void*& slot, const int32_t* done, int (*body)(Problem&), int64_t* body_launches);
void destroy_loop(void*& slot);
void uncount_launches(int64_t n);
void add_launches(int64_t n);
int64_t thread_launch_count();  // launches counted on the calling thread
// exact_sections.cu: the bonds of voxel-face interfaces (bad: device counter of sections whose
// indices lie outside the arrays, or null)
int build_bonds_device(const svxg_node* nodes, int32_t n, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                       int64_t nf, const svxg_junction* juncs, int64_t nj, const svxg_lattice* lats, int32_t nl,
                       int32_t samples, const svxg_material* mats, svxg_bond* out, int32_t* bad, cudaStream_t st);
// scan.cu
int exclusive_scan_i32(Problem& P, const int32_t* in, int32_t* out, int64_t n, int32_t* total_host);
const int32_t* scan_total_device(const Problem& P, int64_t n);  // the last scan's total (device)
// exact_cascade.cu: the judge's break rounds (the host loop: svxg_cascade, capi.cu)
struct CascadeState {  // device; the host reads it once or twice a round
  int32_t m;          // bonds at or over strength
  int32_t K;          // bonds the round breaks
  int32_t n_thr;      // bonds at or over the round's threshold
  int32_t any_in_k;   // a removed bond was in K
  int32_t r;          // nodes no support holds
  int32_t rb;         // bonds of those nodes
  int32_t r_dof;      // a retired node had a free DOF
  int32_t pad;
  double top;         // the largest phi over strength
  unsigned long long maxphi_bits;  // the largest phi of the judgement
  double spent;       // fracture energy paid so far (pieces)
  int32_t poor;       // the energy ran out this round (pieces)
  int32_t pad2;
};
// How a round picks its breaks: a structure's (fraction < 0: at least the worst quarter, no
// energy) or a piece's (at least ceil(fraction x m); energy >= 0: cracks paid from it)
struct BreakRule {
  double fraction = -1.0;
  double energy = -1.0;
  double spent = 0.0;
  double fracture_energy = 1.0, crush_energy = 20.0;
  const double* gf = nullptr;  // device, Gf per material
};
struct CascadeScratch {
  char* base = nullptr;
  cudaStream_t stream = nullptr;
  CascadeState* st = nullptr;
  double *u = nullptr, *f = nullptr, *u0 = nullptr;  // node order, 6 per node
  svxg_bond_load* judged = nullptr;
  uint8_t* has = nullptr;
  double* phi = nullptr;
  int32_t *flag = nullptr, *pos = nullptr, *over = nullptr, *sel = nullptr, *blist = nullptr;
  int32_t* parent = nullptr;
  uint8_t *held = nullptr, *now = nullptr;
  int32_t *nlist = nullptr, *npos = nullptr;
  unsigned long long* gphi = nullptr;
  int32_t* gb = nullptr;
  int64_t gcap = 0;
  uint8_t *broken8 = nullptr, *in_k8 = nullptr;
  uint8_t *mode = nullptr, *selmode = nullptr;
  double* gf = nullptr;
};
int cascade_alloc(Problem& P, CascadeScratch& S, int32_t max_breaks);
void cascade_free(CascadeScratch& S);
int cascade_judge(Problem& P, CascadeScratch& S, double fragility, double dif, int blend, double band,
                  int32_t max_breaks, const BreakRule& rule);
int cascade_roots(Problem& P, CascadeScratch& S);
int cascade_gather_modes(Problem& P, CascadeScratch& S, int32_t count);
int unbreak_list(Problem& P, const int32_t* list_dev, int32_t count);
int cascade_find_loose(Problem& P, CascadeScratch& S);
int cascade_retire(Problem& P, CascadeScratch& S, int32_t r);
int cascade_bond_flags(Problem& P, CascadeScratch& S);
// StressProblem::remove_bond of a device list of distinct bonds, in list order (count: *count_dev
// if given, else bound); unassembled: the bonds only break
int remove_bonds_list(Problem& P, const int32_t* list, const int32_t* count_dev, int32_t bound, CascadeState* st);

}  // namespace svxg
