// capi.cu - the C ABI (include/svxg.h): svx::StressProblem's lifecycle over the device state.
//
// Host-side bookkeeping mirrors the reference's members (core/src/stress/stress.cpp): the graph
// is kept on the host as well so that remove_bond / retire_nodes can pick their bonds and rows
// as the reference does; every number is computed on the device.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <mutex>
#include <new>

#include "problem.cuh"

struct svxg_problem {
  svxg::Problem P;
};

namespace svxg {

namespace {
thread_local std::string g_error;

struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~DeviceScope() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

#define TRY(x)            \
  do {                    \
    int e__ = (x);        \
    if (e__) return e__;  \
  } while (0)

#define CHECK_P(p)                              \
  do {                                          \
    if (!(p)) {                                 \
      set_error("null problem");                \
      return SVXG_ERR_ARG;                      \
    }                                           \
  } while (0)

void release_solver(Problem& P) {
  destroy_loop(P.loop_plain);
  destroy_loop(P.loop_mixed);
  free_run(P);
  release_appended(P);
  P.pc_n = 0;
  P.mem.release(P.K.rowptr);
  P.mem.release(P.K.col);
  P.mem.release(P.K.val);
  P.mem.release(P.K.val32);
  P.K = Bsr{};
  P.mem.release(P.d_kslots);
  P.mem.release(P.d_seg_row);
  P.mem.release(P.d_seg);
  P.mem.release(P.d_seg_flag);
  P.mem.release(P.d_seg_of_row);
  P.mem.release(P.d_seg_lmap);
  P.mem.release(P.d_jinv);
  P.mem.release(P.d_dof);
  P.mem.release(P.d_chol);
  for (Level& L : P.lv) {
    P.mem.release(L.A.rowptr);
    P.mem.release(L.A.col);
    P.mem.release(L.A.val);
    P.mem.release(L.A.val32);
    P.mem.release(L.dinv);
    P.mem.release(L.dinv32);
    P.mem.release(L.parent);
    P.mem.release(L.pos);
    P.mem.release(L.prow);
    P.mem.release(L.pcol);
    P.mem.release(L.pval);
    P.mem.release(L.pval32);
    P.mem.release(L.rrow);
    P.mem.release(L.rent_i);
    P.mem.release(L.rent_e);
    P.mem.release(L.b32);
    P.mem.release(L.x32);
    P.mem.release(L.r32);
    P.mem.release(L.t32);
    P.mem.release(L.u32);
  }
  P.mem.release(P.d_cinv);
  P.mem.release(P.d_cvec);
  P.mem.release(P.d_rm_head);
  P.rm_head_cap = 0;
  P.mem.release(P.d_cinv32);
  {
    char* bd = static_cast<char*>(P.d_bdesc);
    P.mem.release(bd);
    P.d_bdesc = nullptr;
  }
  P.lv.clear();
  P.chol_n = 0;
  P.amg_work = P.amg_build_work = 0;
  P.assembled = false;
  P.pc_current = false;
  P.jacobi_only = false;
  P.nfree = 0;
  P.h_dof.clear();
}

int upload_bond_flags(Problem& P, int32_t b) {
  // (broken and in_k of one bond -> the device record; synchronous: the bytes are on the stack)
  const uint8_t flags[2] = {P.h_broken[size_t(b)], P.h_in_k[size_t(b)]};
  static_assert(offsetof(svxg_bond, in_k) == offsetof(svxg_bond, broken) + 1, "flag bytes adjacent");
  SVXG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(P.d_bonds + b) + offsetof(svxg_bond, broken), flags, 2,
                            cudaMemcpyHostToDevice, P.stream));
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

}  // namespace

void set_error(const std::string& msg) { g_error = msg; }

// More hardware work queues than the driver's default of 8: a server's slots (and hosts that solve
// on many threads) run a stream each, and streams beyond the queue count share queues and
// serialize (the loose-pieces batch ran at half its rate with 8). The driver reads the variable
// when the process's CUDA context is made, so it is set when the library loads, unless the host
// chose a value; a context made before the library loaded keeps its own.
__attribute__((constructor)) static void default_connections() { setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0); }

namespace {
std::atomic<int64_t> g_launches{0};
std::atomic<int64_t> g_graph_launches{0};  // (the part of g_launches run inside loop graphs)
thread_local int64_t t_launches = 0;       // (this thread's: what a capture on it enqueued)
}
void count_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  ++t_launches;
}
int64_t thread_launch_count() { return t_launches; }
void uncount_launches(int64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }
void add_launches(int64_t n) {
  g_launches.fetch_add(n, std::memory_order_relaxed);
  g_graph_launches.fetch_add(n, std::memory_order_relaxed);
}

namespace {

constexpr int kPoolDevices = 64;
std::mutex g_pool_mu;

// The library's pool on `dev`: it keeps what is freed (no release threshold), and it never makes
// one stream wait for another to reuse memory (a stream reuses only what its own order, or a
// finished free, allows), so concurrent problems do not serialize through the allocator.
// One pool per device and host thread: concurrent problems on other threads (a server's slots)
// allocate and free without contending for one pool's lock. Memory freed by a thread returns to
// the pool of the thread that allocated it.
struct ThreadPools {
  cudaMemPool_t pool[kPoolDevices] = {};
  ~ThreadPools() {
    // (outstanding allocations keep a destroyed pool's memory until they are freed)
    for (cudaMemPool_t& p : pool)
      if (p) cudaMemPoolDestroy(p);
  }
};
thread_local ThreadPools t_pools;

cudaError_t library_pool(int dev, cudaMemPool_t* out) {
  if (dev < 0 || dev >= kPoolDevices) return cudaErrorInvalidDevice;
  if (t_pools.pool[dev]) {
    *out = t_pools.pool[dev];
    return cudaSuccess;
  }
  std::lock_guard<std::mutex> lk(g_pool_mu);
  {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    int no = 0;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return e;
    }
    t_pools.pool[dev] = pool;
  }
  *out = t_pools.pool[dev];
  return cudaSuccess;
}

}  // namespace

namespace {

std::atomic<int> g_blocking{[] {
  const char* v = std::getenv("SVXG_BLOCKING_SYNC");
  return v && v[0] && v[0] != '0' ? 1 : 0;
}()};

// one blocking-sync event per host thread (and device)
struct WaitEvent {
  cudaEvent_t ev = nullptr;
  int device = -1;
  ~WaitEvent() {
    if (ev) cudaEventDestroy(ev);
  }
};
thread_local WaitEvent t_wait;

}  // namespace

// SVXG_BLOCKING_SYNC=0 keeps spinning waits even under a server (=1 forces sleeping waits)
const int g_blocking_env = [] {
  const char* v = std::getenv("SVXG_BLOCKING_SYNC");
  return v && v[0] ? (v[0] == '0' ? 0 : 1) : -1;
}();

void blocking_waits(bool on) {
  if (g_blocking_env == 0) return;
  g_blocking.fetch_add(on ? 1 : -1);
}

cudaError_t host_wait(cudaStream_t s) {
  if (g_blocking.load(std::memory_order_relaxed) <= 0) return cudaStreamSynchronize(s);
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (!t_wait.ev || t_wait.device != dev) {
    if (t_wait.ev) cudaEventDestroy(t_wait.ev);
    t_wait.ev = nullptr;
    e = cudaEventCreateWithFlags(&t_wait.ev, cudaEventBlockingSync | cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    t_wait.device = dev;
  }
  e = cudaEventRecord(t_wait.ev, s);
  if (e != cudaSuccess) return e;
  return cudaEventSynchronize(t_wait.ev);
}

// The calling thread's pool on the current device keeps at most `keep` bytes it is not using
// (a server slot calls this after each request, so one large request does not leave its peak
// reserved for good).
void pool_trim(size_t keep) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kPoolDevices) {
    cudaGetLastError();
    return;
  }
  if (t_pools.pool[dev]) cudaMemPoolTrimTo(t_pools.pool[dev], keep);
}

cudaError_t pool_malloc_async(void** p, size_t bytes, cudaStream_t s) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaMemPool_t pool = nullptr;
  e = library_pool(dev, &pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

}  // namespace svxg

using namespace svxg;

namespace svxg {

int ensure_node_vectors(Problem& P) {
  if (!P.d_un) TRY(P.mem.alloc(&P.d_un, 12 * size_t(std::max(P.n, 1))));  // u, then f
  if (!P.mem.holds(P.d_un, 12 * sizeof(double) * size_t(std::max(P.n, 1)))) {
    set_error("node vectors: buffer does not hold 12 n doubles");
    return SVXG_ERR_STATE;
  }
  return SVXG_OK;
}

}  // namespace svxg

extern "C" {

const char* svxg_last_error(void) { return g_error.c_str(); }

int64_t svxg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }
int64_t svxg_graph_launch_count(void) { return g_graph_launches.load(std::memory_order_relaxed); }

int svxg_timer_enable(svxg_problem* p, int32_t on) {
  CHECK_P(p);
  p->P.timer_on = on != 0;
  p->P.timer_kind = SVXG_TIMER_CG_SPMV;
  return SVXG_OK;
}

int svxg_timer_enable_kernel(svxg_problem* p, int32_t kind, int32_t on) {
  CHECK_P(p);
  if (kind != SVXG_TIMER_CG_SPMV && kind != SVXG_TIMER_GALERKIN_AP) {
    set_error("svxg_timer_enable_kernel: unknown kernel");
    return SVXG_ERR_ARG;
  }
  p->P.timer_on = on != 0;
  p->P.timer_kind = kind;
  p->P.timer_used = 0;
  p->P.timer_work = 0;
  return SVXG_OK;
}

int svxg_timer_read_work(svxg_problem* p, double* ms_total, int64_t* launches, int64_t* work) {
  CHECK_P(p);
  const int64_t w = p->P.timer_work;
  const int e = svxg_timer_read(p, ms_total, launches);
  if (e) return e;
  if (work) *work = w;
  p->P.timer_work = 0;
  return SVXG_OK;
}

int svxg_phase_timing(svxg_problem* p, int32_t on) {
  CHECK_P(p);
  p->P.phase_on = on != 0;
  p->P.phase_used = 0;
  return SVXG_OK;
}

int svxg_phase_times(svxg_problem* p, svxg_phase_time* out, int32_t cap, int32_t* count) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  SVXG_CUDA(host_wait(P.stream));
  const int32_t n = P.phase_used > 1 ? int32_t(P.phase_used - 1) : 0;
  if (count) *count = n;
  for (int32_t i = 0; out && i < std::min(n, cap); ++i) {
    float ms = 0.0f;
    SVXG_CUDA(cudaEventElapsedTime(&ms, P.phase_events[size_t(i)], P.phase_events[size_t(i) + 1]));
    out[i].ms = ms;
    std::memset(out[i].label, 0, sizeof(out[i].label));
    const char* l = P.phase_labels[size_t(i) + 1];
    std::strncpy(out[i].label, l ? l : "", sizeof(out[i].label) - 1);
  }
  return SVXG_OK;
}

int svxg_timer_read(svxg_problem* p, double* ms_total, int64_t* launches) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  SVXG_CUDA(host_wait(P.stream));
  double tot = 0.0;
  for (size_t k = 0; k + 1 < 2 * P.timer_used + 1 && k / 2 < P.timer_used; k += 2) {
    float ms = 0.0f;
    SVXG_CUDA(cudaEventElapsedTime(&ms, P.timer_events[k], P.timer_events[k + 1]));
    tot += ms;
  }
  if (ms_total) *ms_total = tot;
  if (launches) *launches = int64_t(P.timer_used);
  P.timer_used = 0;
  return SVXG_OK;
}

int svxg_time_spmv(svxg_problem* p, int32_t precision, int32_t reps, double* ms_per_launch) {
  CHECK_P(p);
  if (!ms_per_launch || reps <= 0) return SVXG_ERR_ARG;
  Problem& P = p->P;
  if (!P.assembled) {
    set_error("svxg_time_spmv: not assembled");
    return SVXG_ERR_STATE;
  }
  DeviceScope ds(P.device);
  float ms = 0.0f;
  if (precision == SVXG_PRECISION_FP64) {
    TRY(time_cg_spmv(P, reps, &ms));
  } else {
    if (!P.K.val32) {
      set_error("svxg_time_spmv: no FP32 copy of K (block-Jacobi problem)");
      return SVXG_ERR_STATE;
    }
    TRY(time_cg_spmv32(P, reps, &ms));
  }
  *ms_per_launch = double(ms);
  return SVXG_OK;
}

int svxg_measure_fp64_rate(int device, double* tflops) {
  if (!tflops) return SVXG_ERR_ARG;
  return measure_fp64_rate(device, tflops);
}

int svxg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int svxg_problem_create(svxg_problem** out, int device) {
  if (!out) return SVXG_ERR_ARG;
  *out = nullptr;
  if (svxg_device_count() <= device || device < 0) {
    set_error("no such CUDA device");
    return SVXG_ERR_NODEVICE;
  }
  DeviceScope ds(device);
  svxg_problem* p = new (std::nothrow) svxg_problem;
  if (!p) return SVXG_ERR_NOMEM;
  p->P.device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&p->P.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    delete p;
    return SVXG_ERR_CUDA;
  }
  p->P.mem.stream = p->P.stream;
  p->P.opt = svxg_default_options();
  *out = p;
  return SVXG_OK;
}

void svxg_problem_destroy(svxg_problem* p) {
  if (!p) return;
  DeviceScope ds(p->P.device);
  destroy_loop(p->P.loop_plain);
  destroy_loop(p->P.loop_mixed);
  p->P.mem.release_all();
  host_wait(p->P.stream);
  for (cudaEvent_t e : p->P.timer_events) cudaEventDestroy(e);
  for (cudaEvent_t e : p->P.phase_events) cudaEventDestroy(e);
  if (!p->P.borrowed) {
    if (p->P.h_s) cudaFreeHost(p->P.h_s);
    if (p->P.h_ms) cudaFreeHost(p->P.h_ms);
    cudaStreamDestroy(p->P.stream);
  }
  delete p;
}

void* svxg_problem_stream(svxg_problem* p) { return p ? static_cast<void*>(p->P.stream) : nullptr; }

}  // extern "C"

namespace svxg {

static int check_graph(const char* who, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                       const svxg_material* mats) {
  if (n < 0 || nb < 0 || (n > 0 && !nodes) || (nb > 0 && !bonds) || !mats) {
    set_error(std::string(who) + ": bad sizes or null arrays");
    return SVXG_ERR_ARG;
  }
  for (int32_t k = 0; k < nb; ++k) {
    const svxg_bond& b = bonds[k];
    if (b.a < 0 || b.a >= n || b.b >= n || b.b == b.a || b.ma >= SVXG_MAX_MATERIALS || b.mb >= SVXG_MAX_MATERIALS) {
      set_error(std::string(who) + ": bond " + std::to_string(k) + " has a bad node or material");
      return SVXG_ERR_ARG;
    }
  }
  return SVXG_OK;
}

// the graph's device and host copies replaced (the solver is left as it is)
static int upload_graph(Problem& P, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                        const svxg_material* mats) {
  P.seg_n = 0;  // (one graph; svxg_set_graphs makes a batch after this)
  P.seg_node.clear();
  P.seg_bond.clear();
  P.mem.release(P.d_nodes);
  P.mem.release(P.d_bonds);
  P.mem.release(P.d_mats);
  P.mem.release(P.d_un);
  P.n = n;
  P.nb = nb;
  P.h_nodes.assign(nodes, nodes + n);
  P.h_bond_ab.resize(2 * size_t(nb));
  P.h_broken.resize(size_t(nb));
  P.h_in_k.resize(size_t(nb));
  for (int32_t k = 0; k < nb; ++k) {
    P.h_bond_ab[2 * size_t(k)] = bonds[k].a;
    P.h_bond_ab[2 * size_t(k) + 1] = bonds[k].b;
    P.h_broken[size_t(k)] = bonds[k].broken;
    P.h_in_k[size_t(k)] = bonds[k].in_k;
  }
  P.h_mats.assign(mats, mats + SVXG_MAX_MATERIALS);
  TRY(P.mem.alloc(&P.d_nodes, size_t(n)));
  TRY(P.mem.alloc(&P.d_bonds, size_t(nb)));
  TRY(P.mem.alloc(&P.d_mats, size_t(SVXG_MAX_MATERIALS)));
  if (n) SVXG_CUDA(cudaMemcpyAsync(P.d_nodes, nodes, sizeof(svxg_node) * size_t(n), cudaMemcpyHostToDevice, P.stream));
  if (nb) SVXG_CUDA(cudaMemcpyAsync(P.d_bonds, bonds, sizeof(svxg_bond) * size_t(nb), cudaMemcpyHostToDevice, P.stream));
  SVXG_CUDA(cudaMemcpyAsync(P.d_mats, mats, sizeof(svxg_material) * SVXG_MAX_MATERIALS, cudaMemcpyHostToDevice,
                            P.stream));
  SVXG_CUDA(host_wait(P.stream));
  P.have_graph = true;
  return SVXG_OK;
}

// A device-resident graph's bookkeeping: each bond's nodes and flags for the host copies, and the
// lowest index of a bond with a bad node or material (atomicMin: the same index whatever the order)
__global__ void k_graph_book(int32_t n, int32_t nb, const svxg_bond* __restrict__ bonds, int32_t* ab, uint8_t* broken,
                             uint8_t* in_k, int32_t* bad) {
  const int64_t k = int64_t(blockIdx.x) * 256 + threadIdx.x;
  if (k >= nb) return;
  const svxg_bond b = bonds[k];
  ab[2 * k] = b.a;
  ab[2 * k + 1] = b.b;
  broken[k] = b.broken;
  in_k[k] = b.in_k;
  if (b.a < 0 || b.a >= n || b.b >= n || b.b == b.a || b.ma >= SVXG_MAX_MATERIALS || b.mb >= SVXG_MAX_MATERIALS)
    atomicMin(bad, int32_t(k));
}

// Bond node indices of a batch moved by their graph's node offset: bond k of graph g (bonds
// [boff[g], boff[g + 1])) gets noff[g] added to a, and to b unless it is a support (-1).
__global__ void k_batch_offsets(int32_t nb, int32_t count, const int64_t* __restrict__ boff,
                                const int64_t* __restrict__ noff, svxg_bond* bonds) {
  const int64_t k = int64_t(blockIdx.x) * 256 + threadIdx.x;
  if (k >= nb) return;
  int32_t lo = 0, hi = count - 1;  // (the last g with boff[g] <= k)
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) / 2;
    if (boff[mid] <= k) lo = mid;
    else hi = mid - 1;
  }
  const int32_t o = int32_t(noff[lo]);
  bonds[k].a += o;
  if (bonds[k].b >= 0) bonds[k].b += o;
}

// the graph's host bookkeeping read back from its device copies (nodes, each bond's nodes and
// flags, the materials); a bond with a bad node or material: SVXG_ERR_ARG, no graph
static int finish_device_graph(Problem& P, const char* who) {
  const int32_t n = P.n, nb = P.nb;
  cudaStream_t st = P.stream;
  // scratch: the bad index, a b pairs, broken, in_k
  const size_t bytes = sizeof(int32_t) * (2 * size_t(nb) + 1) + 2 * size_t(nb) + 16;
  char* tmp = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&tmp), bytes, st));
  int32_t* d_bad = reinterpret_cast<int32_t*>(tmp);
  int32_t* d_ab = d_bad + 1;
  uint8_t* d_broken = reinterpret_cast<uint8_t*>(d_ab + 2 * size_t(nb));
  uint8_t* d_ink = d_broken + nb;
  SVXG_CUDA(cudaMemsetAsync(d_bad, 0x7f, sizeof(int32_t), st));
  if (nb)
    (k_graph_book<<<unsigned((int64_t(nb) + 255) / 256), 256, 0, st>>>(n, nb, P.d_bonds, d_ab, d_broken, d_ink, d_bad),
     SVXG_COUNT_LAUNCH());
  SVXG_CUDA(cudaGetLastError());
  P.h_nodes.resize(size_t(n));
  P.h_bond_ab.resize(2 * size_t(nb));
  P.h_broken.resize(size_t(nb));
  P.h_in_k.resize(size_t(nb));
  P.h_mats.resize(SVXG_MAX_MATERIALS);
  int32_t bad = 0;
  if (n) SVXG_CUDA(cudaMemcpyAsync(P.h_nodes.data(), P.d_nodes, sizeof(svxg_node) * size_t(n), cudaMemcpyDeviceToHost, st));
  if (nb) {
    SVXG_CUDA(cudaMemcpyAsync(P.h_bond_ab.data(), d_ab, sizeof(int32_t) * 2 * size_t(nb), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(cudaMemcpyAsync(P.h_broken.data(), d_broken, size_t(nb), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(cudaMemcpyAsync(P.h_in_k.data(), d_ink, size_t(nb), cudaMemcpyDeviceToHost, st));
  }
  SVXG_CUDA(cudaMemcpyAsync(P.h_mats.data(), P.d_mats, sizeof(svxg_material) * SVXG_MAX_MATERIALS,
                            cudaMemcpyDeviceToHost, st));
  SVXG_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  cudaFreeAsync(tmp, st);
  SVXG_CUDA(host_wait(st));
  if (bad < nb) {
    set_error(std::string(who) + ": bond " + std::to_string(bad) + " has a bad node or material");
    P.mem.release(P.d_nodes);
    P.mem.release(P.d_bonds);
    P.mem.release(P.d_mats);
    P.n = P.nb = 0;
    P.seg_n = 0;
    P.seg_node.clear();
    P.seg_bond.clear();
    return SVXG_ERR_ARG;
  }
  P.have_graph = true;
  return SVXG_OK;
}

// The graphs' device copies from device arrays (one graph: count 1; a batch: graph g after those
// before it, its bonds' node indices moved by its node offset), then the host bookkeeping.
static int upload_graphs_device(Problem& P, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                                const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats) {
  P.seg_n = 0;
  P.seg_node.clear();
  P.seg_bond.clear();
  P.mem.release(P.d_nodes);
  P.mem.release(P.d_bonds);
  P.mem.release(P.d_mats);
  P.mem.release(P.d_un);
  P.have_graph = false;
  std::vector<int64_t> so(size_t(count) + 1, 0), sb(size_t(count) + 1, 0);
  for (int32_t g = 0; g < count; ++g) {
    so[size_t(g) + 1] = so[size_t(g)] + n[g];
    sb[size_t(g) + 1] = sb[size_t(g)] + nb[g];
  }
  if (so.back() > INT32_MAX || sb.back() > INT32_MAX) {
    set_error("set_graphs: more than 2^31 nodes or bonds in all");
    return SVXG_ERR_ARG;
  }
  P.n = int32_t(so.back());
  P.nb = int32_t(sb.back());
  TRY(P.mem.alloc(&P.d_nodes, size_t(P.n)));
  TRY(P.mem.alloc(&P.d_bonds, size_t(P.nb)));
  TRY(P.mem.alloc(&P.d_mats, size_t(SVXG_MAX_MATERIALS)));
  cudaStream_t st = P.stream;
  for (int32_t g = 0; g < count; ++g) {
    if (n[g])
      SVXG_CUDA(cudaMemcpyAsync(P.d_nodes + so[size_t(g)], nodes[g], sizeof(svxg_node) * size_t(n[g]),
                                cudaMemcpyDeviceToDevice, st));
    if (nb[g])
      SVXG_CUDA(cudaMemcpyAsync(P.d_bonds + sb[size_t(g)], bonds[g], sizeof(svxg_bond) * size_t(nb[g]),
                                cudaMemcpyDeviceToDevice, st));
  }
  SVXG_CUDA(cudaMemcpyAsync(P.d_mats, mats, sizeof(svxg_material) * SVXG_MAX_MATERIALS, cudaMemcpyDeviceToDevice,
                            st));
  if (count > 1 && P.nb > 0) {
    int64_t* off = nullptr;
    SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&off), sizeof(int64_t) * 2 * (size_t(count) + 1), st));
    SVXG_CUDA(cudaMemcpyAsync(off, sb.data(), sizeof(int64_t) * sb.size(), cudaMemcpyHostToDevice, st));
    SVXG_CUDA(cudaMemcpyAsync(off + count + 1, so.data(), sizeof(int64_t) * so.size(), cudaMemcpyHostToDevice, st));
    (k_batch_offsets<<<unsigned((int64_t(P.nb) + 255) / 256), 256, 0, st>>>(P.nb, count, off, off + count + 1,
                                                                              P.d_bonds),
     SVXG_COUNT_LAUNCH());
    cudaFreeAsync(off, st);
    SVXG_CUDA(host_wait(st));  // (so and sb are host vectors read by the copies above)
  }
  TRY(finish_device_graph(P, count > 1 ? "svxg_set_graphs_device" : "svxg_set_graph_device"));
  if (count > 1) {
    P.seg_n = count;
    P.seg_node = std::move(so);
    P.seg_bond = std::move(sb);
  }
  return SVXG_OK;
}

}  // namespace svxg

extern "C" {

int svxg_set_graph_device(svxg_problem* p, const svxg_node* nodes_dev, int32_t n, const svxg_bond* bonds_dev,
                          int32_t nb, const svxg_material* mats_dev) {
  CHECK_P(p);
  if (n < 0 || nb < 0 || (n > 0 && !nodes_dev) || (nb > 0 && !bonds_dev) || !mats_dev) {
    set_error("svxg_set_graph_device: bad sizes or null arrays");
    return SVXG_ERR_ARG;
  }
  Problem& P = p->P;
  DeviceScope ds(P.device);
  release_solver(P);
  return upload_graphs_device(P, 1, &nodes_dev, &n, &bonds_dev, &nb, mats_dev);
}

int svxg_set_graphs_device(svxg_problem* p, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                           const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats) {
  CHECK_P(p);
  if (count < 1 || !nodes || !n || !bonds || !nb || !mats) {
    set_error("svxg_set_graphs_device: bad count or null arrays");
    return SVXG_ERR_ARG;
  }
  for (int32_t g = 0; g < count; ++g)
    if (n[g] < 0 || nb[g] < 0 || (n[g] > 0 && !nodes[g]) || (nb[g] > 0 && !bonds[g])) {
      set_error("svxg_set_graphs_device: graph " + std::to_string(g) + " has bad sizes or null arrays");
      return SVXG_ERR_ARG;
    }
  Problem& P = p->P;
  DeviceScope ds(P.device);
  release_solver(P);
  return upload_graphs_device(P, count, nodes, n, bonds, nb, mats);
}

int svxg_set_graphs(svxg_problem* p, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                    const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats) {
  CHECK_P(p);
  if (count < 1 || !nodes || !n || !bonds || !nb || !mats) {
    set_error("svxg_set_graphs: bad count or null arrays");
    return SVXG_ERR_ARG;
  }
  int64_t tn = 0, tb = 0;
  for (int32_t g = 0; g < count; ++g) {
    TRY(check_graph("svxg_set_graphs", nodes[g], n[g], bonds[g], nb[g], mats));
    tn += n[g];
    tb += nb[g];
  }
  if (tn > INT32_MAX || tb > INT32_MAX) {
    set_error("svxg_set_graphs: more than 2^31 nodes or bonds in all");
    return SVXG_ERR_ARG;
  }
  // one graph of them all: graph g's nodes and bonds after those of the graphs before it, its bonds'
  // node indices moved by its node offset (supports stay -1)
  std::vector<svxg_node> un(static_cast<size_t>(tn));
  std::vector<svxg_bond> ub(static_cast<size_t>(tb));
  std::vector<int64_t> so(size_t(count) + 1, 0), sb(size_t(count) + 1, 0);
  for (int32_t g = 0; g < count; ++g) {
    const int64_t o = so[size_t(g)], ob = sb[size_t(g)];
    if (n[g]) std::memcpy(&un[size_t(o)], nodes[g], sizeof(svxg_node) * size_t(n[g]));
    for (int32_t k = 0; k < nb[g]; ++k) {
      svxg_bond b = bonds[g][k];
      b.a += int32_t(o);
      if (b.b >= 0) b.b += int32_t(o);
      ub[size_t(ob + k)] = b;
    }
    so[size_t(g) + 1] = o + n[g];
    sb[size_t(g) + 1] = ob + nb[g];
  }
  Problem& P = p->P;
  DeviceScope ds(P.device);
  release_solver(P);
  TRY(upload_graph(P, un.data(), int32_t(tn), ub.data(), int32_t(tb), mats));
  if (count > 1) {
    P.seg_n = count;
    P.seg_node = std::move(so);
    P.seg_bond = std::move(sb);
  }
  return SVXG_OK;
}

int svxg_graph_results(svxg_problem* p, int32_t count, double* rel_res, int32_t* converged, int32_t* iters,
                       double* err_est) {
  CHECK_P(p);
  Problem& P = p->P;
  if (P.seg_n <= 0 || count != P.seg_n) {
    set_error("svxg_graph_results: not a batch of that many graphs");
    return SVXG_ERR_ARG;
  }
  if (!P.d_seg) {
    set_error("svxg_graph_results: not assembled");
    return SVXG_ERR_STATE;
  }
  DeviceScope ds(P.device);
  return seg_results(P, rel_res, converged, iters, err_est);
}

int svxg_set_graph(svxg_problem* p, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                   const svxg_material* mats) {
  CHECK_P(p);
  Problem& P = p->P;
  TRY(check_graph("svxg_set_graph", nodes, n, bonds, nb, mats));
  DeviceScope ds(P.device);
  release_solver(P);
  return upload_graph(P, nodes, n, bonds, nb, mats);
}

static int assemble_impl(Problem& P, const svxg_stress_options* opt, int32_t* ok) {
  if (ok) *ok = 0;
  if (!P.have_graph) {
    set_error("svxg_assemble: no graph");
    return SVXG_ERR_STATE;
  }
  DeviceScope ds(P.device);
  P.opt = opt ? *opt : svxg_default_options();
  trace_mark(P, "start", true);
  release_solver(P);
  P.tune_log.clear();
  P.mixed_fallbacks = 0;
  P.host_loops = 0;
  P.pc_current = true;
  TRY(assemble_matrix(P));
  trace_mark(P, "K assembled");
  P.assembly_work = 0;
  P.assembly_work = 48 * int64_t(std::count(P.h_in_k.begin(), P.h_in_k.end(), uint8_t(1)));
  P.jacobi_only = P.nfree < P.opt.amg_min_nodes;
  if (P.jacobi_only) {
    TRY(build_jacobi(P));
    P.assembly_work += 12 * int64_t(P.nfree);
  } else {
    int32_t built = 0;
    TRY(build_multigrid(P, &built));
    if (!built) {
      P.assembled = false;
      return SVXG_OK;
    }
    P.assembly_work += P.amg_build_work;
  }
  trace_mark(P, "preconditioner built");
  TRY(tune_k64(P));
  TRY(seg_prepare(P));
  P.sched_k32 = P.jacobi_only || P.lv.empty() ? 0 : P.lv[0].sched_a;  // (K32 is level 0's cycle operator)
  SVXG_CUDA(host_wait(P.stream));
  P.pc_n = P.jacobi_only ? 0 : P.nfree;
  P.assembled = true;
  if (ok) *ok = 1;
  return SVXG_OK;
}

// StressProblem::reassemble (stress.cpp:178-211) with the graph replaced by the caller's
static int reassemble_impl(Problem& P, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                           const svxg_material* mats, int32_t* ok) {
  if (ok) *ok = 0;
  const svxg_stress_options opt = P.opt;
  if (!P.assembled || P.jacobi_only || P.lv.empty() || P.pc_n == 0) {
    release_solver(P);
    TRY(upload_graph(P, nodes, n, bonds, nb, mats));
    return assemble_impl(P, &opt, ok);
  }
  trace_mark(P, "start", true);
  // the multigrid stays; its level-0 operator keeps the arrays of the K it was built from
  destroy_loop(P.loop_plain);
  destroy_loop(P.loop_mixed);
  free_run(P);
  release_appended(P);
  P.mem.release(P.d_jinv);
  P.mem.release(P.d_un);
  if (P.K.val32 && !P.lv.empty() && P.lv[0].A.val32 != P.K.val32) P.mem.release(P.K.val32);
  P.K = Bsr{};
  P.mem.release(P.d_kslots);
  P.assembled = false;
  P.pc_current = false;
  TRY(upload_graph(P, nodes, n, bonds, nb, mats));
  TRY(assemble_matrix(P));
  if (P.nfree < P.pc_n) {  // (nodes left: the indices moved)
    release_solver(P);
    return assemble_impl(P, &opt, ok);
  }
  TRY(build_jacobi(P));
  TRY(build_appended(P));
  TRY(tune_k64(P));
  P.sched_k32 = 0;
  SVXG_CUDA(host_wait(P.stream));
  trace_mark(P, "reassembled");
  P.assembled = true;
  if (ok) *ok = 1;
  return SVXG_OK;
}

int svxg_assemble(svxg_problem* p, const svxg_stress_options* opt, int32_t* ok) {
  CHECK_P(p);
  return assemble_impl(p->P, opt, ok);
}

int svxg_reassemble(svxg_problem* p, const svxg_node* nodes, int32_t n, const svxg_bond* bonds, int32_t nb,
                    const svxg_material* mats, int32_t* ok) {
  CHECK_P(p);
  TRY(check_graph("svxg_reassemble", nodes, n, bonds, nb, mats));
  DeviceScope ds(p->P.device);
  return reassemble_impl(p->P, nodes, n, bonds, nb, mats, ok);
}

int32_t svxg_appended(const svxg_problem* p) {
  return p && p->P.assembled && !p->P.jacobi_only ? p->P.nfree - p->P.pc_n : 0;
}

int svxg_extend_warm_start(svxg_problem* p, double* u, int32_t first_new) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!u) return SVXG_ERR_ARG;
  if (first_new < 0 || first_new >= P.n) return SVXG_OK;
  DeviceScope ds(P.device);
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  SVXG_CUDA(cudaMemcpyAsync(P.d_un, u, m * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  TRY(extend_warm_start_device(P, P.d_un, first_new));
  SVXG_CUDA(cudaMemcpyAsync(u, P.d_un, m * sizeof(double), cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

int svxg_assembled(const svxg_problem* p) { return p && p->P.assembled ? 1 : 0; }

int svxg_invalidate(svxg_problem* p) {
  CHECK_P(p);
  p->P.assembled = false;
  p->P.active = false;
  return SVXG_OK;
}

int svxg_preconditioner_current(const svxg_problem* p) { return p && p->P.assembled && p->P.pc_current ? 1 : 0; }
int svxg_block_jacobi(const svxg_problem* p) { return p && p->P.jacobi_only ? 1 : 0; }

int svxg_release(svxg_problem* p) {
  CHECK_P(p);
  DeviceScope ds(p->P.device);
  host_wait(p->P.stream);
  release_solver(p->P);
  std::fill(p->P.h_in_k.begin(), p->P.h_in_k.end(), uint8_t(0));
  return SVXG_OK;
}

int svxg_remove_bond(svxg_problem* p, int32_t b) {
  CHECK_P(p);
  Problem& P = p->P;
  if (b < 0 || b >= P.nb) {
    set_error("svxg_remove_bond: no such bond");
    return SVXG_ERR_ARG;
  }
  DeviceScope ds(P.device);
  P.h_broken[size_t(b)] = 1;
  if (!P.assembled || !P.h_in_k[size_t(b)]) {
    TRY(upload_bond_flags(P, b));
    SVXG_CUDA(host_wait(P.stream));
    return SVXG_OK;
  }
  P.h_in_k[size_t(b)] = 0;
  TRY(remove_bonds_device(P, &b, 1));
  if (!P.jacobi_only) P.pc_current = false;
  P.active = false;
  return SVXG_OK;
}

// remove_bond of each listed bond in list order, with one device pass and one wait
int svxg_remove_bonds(svxg_problem* p, const int32_t* list, int32_t count) {
  CHECK_P(p);
  Problem& P = p->P;
  if (count <= 0) return SVXG_OK;
  if (!list) return SVXG_ERR_ARG;
  for (int32_t t = 0; t < count; ++t)
    if (list[t] < 0 || list[t] >= P.nb) {
      set_error("svxg_remove_bonds: no such bond");
      return SVXG_ERR_ARG;
    }
  DeviceScope ds(P.device);
  std::vector<int32_t> rm;
  rm.reserve(size_t(count));
  for (int32_t t = 0; t < count; ++t) {
    const int32_t b = list[t];
    P.h_broken[size_t(b)] = 1;
    if (!P.assembled || !P.h_in_k[size_t(b)]) {
      TRY(upload_bond_flags(P, b));  // (not in K: the bond only breaks)
      continue;
    }
    P.h_in_k[size_t(b)] = 0;  // (a repeat of the bond later in the list is then a no-op, as the reference's)
    rm.push_back(b);
  }
  if (!rm.empty()) {
    TRY(remove_bonds_device(P, rm.data(), int32_t(rm.size())));
    if (!P.jacobi_only) P.pc_current = false;
  }
  P.active = false;
  return SVXG_OK;
}

int svxg_retire_nodes(svxg_problem* p, const int32_t* list, int32_t count) {
  CHECK_P(p);
  Problem& P = p->P;
  if (count <= 0) return SVXG_OK;
  for (int32_t t = 0; t < count; ++t)
    if (list[t] < 0 || list[t] >= P.n) {
      set_error("svxg_retire_nodes: no such node");
      return SVXG_ERR_ARG;
    }
  DeviceScope ds(P.device);
  std::vector<uint8_t> now(size_t(P.n), 0);
  for (int32_t t = 0; t < count; ++t) {
    const int32_t i = list[t];
    now[size_t(i)] = P.h_nodes[size_t(i)].gone ? 0 : 1;
    P.h_nodes[size_t(i)].gone = 1;
    SVXG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(P.d_nodes + i) + offsetof(svxg_node, gone), &P.h_nodes[size_t(i)].gone,
                              1, cudaMemcpyHostToDevice, P.stream));
  }
  std::vector<int32_t> rm;
  for (int32_t b = 0; b < P.nb; ++b) {
    const int32_t ba = P.h_bond_ab[2 * size_t(b)], bb = P.h_bond_ab[2 * size_t(b) + 1];
    if (!(now[size_t(ba)] || (bb >= 0 && now[size_t(bb)]))) continue;
    P.h_broken[size_t(b)] = 1;
    if (P.assembled && P.h_in_k[size_t(b)]) {
      P.h_in_k[size_t(b)] = 0;
      rm.push_back(b);
      if (!P.jacobi_only) P.pc_current = false;
    } else {
      TRY(upload_bond_flags(P, b));
    }
  }
  if (P.assembled) TRY(remove_bonds_device(P, rm.data(), int32_t(rm.size())));
  if (P.assembled) {
    std::vector<int32_t> rows;
    for (int32_t t = 0; t < count; ++t) {
      const int32_t i = list[t];
      const int32_t d = P.h_dof[size_t(i)];
      if (d < 0) continue;
      if (now[size_t(i)] && !P.jacobi_only) P.pc_current = false;
      rows.push_back(d);
    }
    TRY(set_identity_rows(P, rows.data(), int32_t(rows.size())));
  }
  SVXG_CUDA(host_wait(P.stream));
  P.active = false;
  return SVXG_OK;
}

int svxg_bond_flags(svxg_problem* p, uint8_t* broken, uint8_t* in_k) {
  CHECK_P(p);
  for (int32_t k = 0; k < p->P.nb; ++k) {
    if (broken) broken[k] = p->P.h_broken[size_t(k)];
    if (in_k) in_k[k] = p->P.h_in_k[size_t(k)];
  }
  return SVXG_OK;
}


static int ensure_assembled(Problem& P) {
  if (P.assembled) return SVXG_OK;
  int32_t ok = 0;
  const svxg_stress_options o = P.opt;
  TRY(assemble_impl(P, &o, &ok));
  if (!ok) return 1;  // (singular: the caller reports a breakdown)
  return SVXG_OK;
}

static void failed_result(svxg_pcg_result* res) {
  if (!res) return;
  std::memset(res, 0, sizeof(*res));
  res->rel_res = INFINITY;
  res->breakdown = 1;
}

static int solve_common(Problem& P, const double* f_dev, double* u_dev, double rtol, int32_t maxit, int32_t warm,
                        svxg_pcg_result* res) {
  TRY(pcg_begin(P, f_dev, warm ? u_dev : nullptr));
  trace_mark(P, "solve: begin");
  TRY(pcg_iterate(P, maxit < 0 ? 100000 : maxit, rtol, res));
  trace_mark(P, "solve: iterate");
  // (the mixed-precision policy states each solve's error: the estimate of solve.cu error_estimate)
  P.last_err_est = 0.0;
  if (P.opt.precision != SVXG_PRECISION_FP64 && res && std::isfinite(res->rel_res)) TRY(error_estimate(P));
  TRY(gather_solution(P, u_dev));
  P.active = false;
  return SVXG_OK;
}

}  // extern "C"

namespace svxg {

int solve_nodes_host(Problem& P, const double* f, double* u, double rtol, int32_t maxit, int warm,
                     svxg_pcg_result* res) {
  DeviceScope ds(P.device);
  const int a = ensure_assembled(P);
  if (a < 0) return a;
  if (a > 0) {
    failed_result(res);
    return SVXG_OK;
  }
  const bool resident = warm == kWarmResident && P.d_un && P.mem.holds(P.d_un, 12 * sizeof(double) * size_t(P.n));
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  double* du = P.d_un;
  double* df = P.d_un + m;
  // (f and u may be host or device memory: the copies take their direction from the pointers)
  SVXG_CUDA(cudaMemcpyAsync(df, f, m * sizeof(double), cudaMemcpyDefault, P.stream));
  if (warm == kWarmHost) SVXG_CUDA(cudaMemcpyAsync(du, u, m * sizeof(double), cudaMemcpyDefault, P.stream));
  trace_mark(P, "solve: load copied");
  TRY(solve_common(P, df, du, rtol, maxit, warm == kWarmHost || resident ? 1 : 0, res));
  if (u) SVXG_CUDA(cudaMemcpyAsync(u, du, m * sizeof(double), cudaMemcpyDefault, P.stream));
  SVXG_CUDA(host_wait(P.stream));
  trace_mark(P, "solve: u copied back");
  return SVXG_OK;
}

// A batch's solve with graph g's load read from f[g] (host or device memory, 6 per node); a graph
// with take[g] == 0 keeps the load of the last solve (a repeat of some graphs replaces only theirs;
// take null: every graph's). warm: from the problem's last solution, still on the device. u of
// graph g goes to u_out[g] (host or device memory; u_out or u_out[g] null: not copied).
int batch_solve_loads(Problem& P, const double* const* f, const uint8_t* take, double* const* u_out, double rtol,
                      int32_t maxit, bool warm, svxg_pcg_result* res) {
  DeviceScope ds(P.device);
  if (P.seg_n <= 0) {
    set_error("batch solve: not a batch");
    return SVXG_ERR_STATE;
  }
  const int a = ensure_assembled(P);
  if (a < 0) return a;
  if (a > 0) {
    failed_result(res);
    return SVXG_OK;
  }
  const bool resident = warm && P.d_un && P.mem.holds(P.d_un, 12 * sizeof(double) * size_t(P.n));
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  double* du = P.d_un;
  double* df = P.d_un + m;
  for (int32_t g = 0; g < P.seg_n; ++g) {
    const size_t o = 6 * size_t(P.seg_node[size_t(g)]), len = 6 * size_t(P.seg_node[size_t(g) + 1]) - o;
    if ((!take || take[g]) && len && f[g])
      SVXG_CUDA(cudaMemcpyAsync(df + o, f[g], len * sizeof(double), cudaMemcpyDefault, P.stream));
  }
  TRY(solve_common(P, df, du, rtol, maxit, resident ? 1 : 0, res));
  for (int32_t g = 0; u_out && g < P.seg_n; ++g) {
    const size_t o = 6 * size_t(P.seg_node[size_t(g)]), len = 6 * size_t(P.seg_node[size_t(g) + 1]) - o;
    if (u_out[g] && len)
      SVXG_CUDA(cudaMemcpyAsync(u_out[g], du + o, len * sizeof(double), cudaMemcpyDefault, P.stream));
  }
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

}  // namespace svxg

extern "C" {

int svxg_solve(svxg_problem* p, const double* f, double* u, double rtol, int32_t maxit, int32_t warm,
               svxg_pcg_result* res) {
  CHECK_P(p);
  if (!f || !u) return SVXG_ERR_ARG;
  return solve_nodes_host(p->P, f, u, rtol, maxit, warm ? kWarmHost : kCold, res);
}

int svxg_solve_device(svxg_problem* p, const double* f_dev, double* u_dev, double rtol, int32_t maxit, int32_t warm,
                      svxg_pcg_result* res) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!f_dev || !u_dev) return SVXG_ERR_ARG;
  DeviceScope ds(P.device);
  const int a = ensure_assembled(P);
  if (a < 0) return a;
  if (a > 0) {
    failed_result(res);
    return SVXG_OK;
  }
  TRY(solve_common(P, f_dev, u_dev, rtol, maxit, warm, res));
  return SVXG_OK;
}

int svxg_begin(svxg_problem* p, const double* f, const double* u0) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  P.active = false;
  const int a = ensure_assembled(P);
  if (a) return a < 0 ? a : SVXG_OK;
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  double* du = P.d_un;
  double* df = P.d_un + m;
  SVXG_CUDA(cudaMemcpyAsync(df, f, m * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  if (u0) SVXG_CUDA(cudaMemcpyAsync(du, u0, m * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  TRY(pcg_begin(P, df, u0 ? du : nullptr));
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

int svxg_iterate(svxg_problem* p, int32_t maxit, double rtol, svxg_pcg_result* res) {
  CHECK_P(p);
  DeviceScope ds(p->P.device);
  return pcg_iterate(p->P, maxit, rtol, res);
}

int svxg_running(const svxg_problem* p) { return p && p->P.active ? 1 : 0; }

int svxg_stop(svxg_problem* p) {
  CHECK_P(p);
  p->P.active = false;
  return SVXG_OK;
}

int svxg_current(svxg_problem* p, double* u) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  const size_t m = 6 * size_t(P.n);
  if (!P.d_x || !P.assembled) {
    std::memset(u, 0, m * sizeof(double));
    return SVXG_OK;
  }
  TRY(ensure_node_vectors(P));
  TRY(gather_solution(P, P.d_un));
  SVXG_CUDA(cudaMemcpyAsync(u, P.d_un, m * sizeof(double), cudaMemcpyDeviceToHost, P.stream));
  SVXG_CUDA(host_wait(P.stream));
  return SVXG_OK;
}

int svxg_bond_loads(svxg_problem* p, const double* u, svxg_bond_load* out) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!out) return SVXG_ERR_ARG;
  DeviceScope ds(P.device);
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  if (u) {
    SVXG_CUDA(cudaMemcpyAsync(P.d_un, u, m * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  } else if (P.d_x && P.assembled) {
    TRY(gather_solution(P, P.d_un));
  } else {
    SVXG_CUDA(cudaMemsetAsync(P.d_un, 0, m * sizeof(double), P.stream));
  }
  svxg_bond_load* d = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&d), sizeof(svxg_bond_load) * size_t(std::max(P.nb, 1)), P.stream));
  int e = bond_loads_device(P, P.d_un, d);
  if (!e && P.nb)
    e = cudaMemcpyAsync(out, d, sizeof(svxg_bond_load) * size_t(P.nb), cudaMemcpyDeviceToHost, P.stream) ==
                cudaSuccess
            ? SVXG_OK
            : SVXG_ERR_CUDA;
  cudaFreeAsync(d, P.stream);
  SVXG_CUDA(host_wait(P.stream));
  return e;
}

int svxg_utilization(svxg_problem* p, double fragility, double* phi, uint8_t* mode, int32_t* over, int32_t cap,
                     int32_t* n_over) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  if (P.d_x && P.assembled) {
    TRY(gather_solution(P, P.d_un));
  } else {
    SVXG_CUDA(cudaMemsetAsync(P.d_un, 0, m * sizeof(double), P.stream));
  }
  const size_t nb = size_t(std::max(P.nb, 1));
  double* dphi = nullptr;
  uint8_t* dmode = nullptr;
  int32_t* dover = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&dphi), nb * sizeof(double), P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&dmode), nb, P.stream));
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&dover), nb * sizeof(int32_t), P.stream));
  int32_t cnt = 0;
  int e = utilization_device(P, P.d_un, fragility, dphi, dmode, dover, &cnt);
  if (!e && P.nb) {
    if (phi) cudaMemcpyAsync(phi, dphi, size_t(P.nb) * sizeof(double), cudaMemcpyDeviceToHost, P.stream);
    if (mode) cudaMemcpyAsync(mode, dmode, size_t(P.nb), cudaMemcpyDeviceToHost, P.stream);
    if (over && cnt > 0)
      cudaMemcpyAsync(over, dover, size_t(std::min(cnt, cap)) * sizeof(int32_t), cudaMemcpyDeviceToHost, P.stream);
  }
  cudaFreeAsync(dphi, P.stream);
  cudaFreeAsync(dmode, P.stream);
  cudaFreeAsync(dover, P.stream);
  SVXG_CUDA(host_wait(P.stream));
  if (n_over) *n_over = cnt;
  return e;
}

int svxg_utilization_device(svxg_problem* p, double fragility, double* phi_dev, uint8_t* mode_dev, int32_t* over_dev,
                            int32_t* n_over) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  TRY(ensure_node_vectors(P));
  const size_t m = 6 * size_t(P.n);
  if (P.d_x && P.assembled) {
    TRY(gather_solution(P, P.d_un));
  } else {
    SVXG_CUDA(cudaMemsetAsync(P.d_un, 0, m * sizeof(double), P.stream));
  }
  return utilization_device(P, P.d_un, fragility, phi_dev, mode_dev, over_dev, n_over);
}

int svxg_debug_trace(svxg_problem* p, char* out, int32_t cap) {
  CHECK_P(p);
  std::string text;
  const auto& tr = p->P.trace;
  for (size_t i = 0; i < tr.size(); ++i) {
    char line[160];
    std::snprintf(line, sizeof(line), "%10.1f %10.1f  %s\n", tr[i].second - tr[0].second,
                  i ? tr[i].second - tr[i - 1].second : 0.0, tr[i].first);
    text += line;
  }
  if (out && cap > 0) {
    const size_t k = std::min(text.size(), size_t(cap - 1));
    std::memcpy(out, text.data(), k);
    out[k] = 0;
  }
  return int(text.size());
}

int svxg_debug_tune_log(svxg_problem* p, svxg_tune_entry* out, int32_t cap, int32_t* count) {
  CHECK_P(p);
  const int32_t k = int32_t(p->P.tune_log.size());
  if (count) *count = k;
  for (int32_t i = 0; out && i < std::min(k, cap); ++i) out[i] = p->P.tune_log[size_t(i)];
  return SVXG_OK;
}

int svxg_get_info(svxg_problem* p, svxg_info* info) {
  CHECK_P(p);
  if (!info) return SVXG_ERR_ARG;
  const Problem& P = p->P;
  std::memset(info, 0, sizeof(*info));
  info->nfree = P.nfree;
  info->block_jacobi = P.jacobi_only ? 1 : 0;
  info->levels = int32_t(P.lv.size());
  info->chol_n = P.chol_n;
  for (size_t l = 0; l < P.lv.size() && l < 16; ++l) {
    info->level_sizes[l] = P.lv[l].A.n;
    info->level_blocks[l] = P.lv[l].A.nnzb;
    info->level_blocks[P.lv.size() + l] = P.lv[l].pnnz;
  }
  info->matrix_blocks = P.K.nnzb;
  info->work_per_apply = P.amg_work;
  info->work_per_iteration = 2 * P.K.nnzb + P.amg_work;
  info->assembly_work = P.assembly_work;
  info->build_work = P.amg_build_work;
  info->device_bytes = P.mem.bytes;
  info->precision = P.opt.precision;
  info->mixed_fallbacks = P.mixed_fallbacks;
  info->error_estimate = P.last_err_est;
  if (P.have_graph)
    info->graph_bytes = int64_t(sizeof(svxg_node)) * std::max<int64_t>(P.n, 1) +
                        int64_t(sizeof(svxg_bond)) * std::max<int64_t>(P.nb, 1) +
                        int64_t(sizeof(svxg_material)) * SVXG_MAX_MATERIALS;
  return SVXG_OK;
}

int svxg_debug_matrix(svxg_problem* p, int32_t* nfree, int64_t* nnzb, int32_t* dof, int32_t* rowptr, int32_t* col,
                      double* val, double* id_scale) {
  CHECK_P(p);
  Problem& P = p->P;
  DeviceScope ds(P.device);
  if (nfree) *nfree = P.K.n;
  if (nnzb) *nnzb = P.K.nnzb;
  if (id_scale) *id_scale = P.id_scale;
  if (!P.assembled && !P.K.val) return SVXG_OK;
  if (dof && P.n) SVXG_CUDA(cudaMemcpy(dof, P.d_dof, sizeof(int32_t) * size_t(P.n), cudaMemcpyDeviceToHost));
  if (rowptr) SVXG_CUDA(cudaMemcpy(rowptr, P.K.rowptr, sizeof(int32_t) * (size_t(P.K.n) + 1), cudaMemcpyDeviceToHost));
  if (col && P.K.nnzb) SVXG_CUDA(cudaMemcpy(col, P.K.col, sizeof(int32_t) * size_t(P.K.nnzb), cudaMemcpyDeviceToHost));
  if (val && P.K.nnzb)
    SVXG_CUDA(cudaMemcpy(val, P.K.val, sizeof(double) * 36 * size_t(P.K.nnzb), cudaMemcpyDeviceToHost));
  return SVXG_OK;
}

int svxg_debug_level_dims(svxg_problem* p, int32_t level, int32_t* n, int64_t* nnzb, int64_t* pnnz) {
  CHECK_P(p);
  const Problem& P = p->P;
  if (level < 0 || size_t(level) >= P.lv.size()) return SVXG_ERR_ARG;
  const Level& L = P.lv[size_t(level)];
  if (n) *n = L.A.n;
  if (nnzb) *nnzb = L.A.nnzb;
  if (pnnz) *pnnz = L.pnnz;
  return SVXG_OK;
}

int svxg_debug_level(svxg_problem* p, int32_t level, int32_t* rowptr, int32_t* col, double* val, double* dinv,
                     int32_t* parent, int32_t* prow, int32_t* pcol, double* pval, double* pos, double* lmax) {
  CHECK_P(p);
  Problem& P = p->P;
  if (level < 0 || size_t(level) >= P.lv.size()) return SVXG_ERR_ARG;
  DeviceScope ds(P.device);
  const Level& L = P.lv[size_t(level)];
  const size_t n = size_t(L.A.n);
  auto get = [&](void* dst, const void* src, size_t bytes) -> int {
    if (!dst || !src || bytes == 0) return SVXG_OK;
    SVXG_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return SVXG_OK;
  };
  TRY(get(rowptr, L.A.rowptr, sizeof(int32_t) * (n + 1)));
  TRY(get(col, L.A.col, sizeof(int32_t) * size_t(L.A.nnzb)));
  TRY(get(val, L.A.val, sizeof(double) * 36 * size_t(L.A.nnzb)));
  TRY(get(dinv, L.dinv, sizeof(double) * 36 * n));
  TRY(get(parent, L.parent, sizeof(int32_t) * n));
  TRY(get(prow, L.prow, sizeof(int32_t) * (n + 1)));
  TRY(get(pcol, L.pcol, sizeof(int32_t) * size_t(L.pnnz)));
  TRY(get(pval, L.pval, sizeof(double) * 36 * size_t(L.pnnz)));
  TRY(get(pos, L.pos, sizeof(double) * 3 * n));
  if (lmax) *lmax = L.lmax;
  return SVXG_OK;
}

int svxg_debug_seq_norm(const double* v, int64_t n, double* out) {
  if (n < 0 || (n > 0 && !v) || !out) return SVXG_ERR_ARG;
  double* d = nullptr;
  SVXG_CUDA(cudaMalloc(&d, sizeof(double) * size_t(n + 1)));
  cudaMemcpy(d, v, sizeof(double) * size_t(n), cudaMemcpyHostToDevice);
  int e = debug_seq_norm(0, d, n, d + n);
  if (!e) e = cudaMemcpy(out, d + n, sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess ? SVXG_OK : SVXG_ERR_CUDA;
  cudaFree(d);
  return e;
}

int svxg_debug_apply(svxg_problem* p, const double* x, double* y) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!P.assembled) return SVXG_ERR_STATE;
  DeviceScope ds(P.device);
  const size_t m = 6 * size_t(P.nfree);
  double *dx = nullptr, *dy = nullptr;
  SVXG_CUDA(cudaMalloc(&dx, (m + 1) * sizeof(double)));
  SVXG_CUDA(cudaMalloc(&dy, (m + 1) * sizeof(double)));
  cudaMemcpy(dx, x, m * sizeof(double), cudaMemcpyHostToDevice);
  int e = spmv(P, P.K, dx, dy);
  host_wait(P.stream);
  if (!e) cudaMemcpy(y, dy, m * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  return e;
}

int svxg_debug_precondition(svxg_problem* p, const double* r, double* z) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!P.assembled) return SVXG_ERR_STATE;
  DeviceScope ds(P.device);
  const size_t m = 6 * size_t(P.nfree);
  double *dr = nullptr, *dz = nullptr;
  SVXG_CUDA(cudaMalloc(&dr, (m + 1) * sizeof(double)));
  SVXG_CUDA(cudaMalloc(&dz, (m + 1) * sizeof(double)));
  cudaMemcpy(dr, r, m * sizeof(double), cudaMemcpyHostToDevice);
  int e = precondition(P, dr, dz);
  host_wait(P.stream);
  if (!e) cudaMemcpy(z, dz, m * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(dr);
  cudaFree(dz);
  return e;
}


// The judge's break rounds of one structure (World::Impl::judge, core/src/world/world.cpp:1162-1277;
// the solve restarts of the tick, world.cpp:1041-1110; detach_unsupported, world.cpp:1371-1458).
// Everything per bond and per node runs on the device; the host reads the round's counts.
int svxg_cascade(svxg_problem* p, const svxg_stress_options* opt, const svxg_cascade_options* co, const double* f,
                 double* u, svxg_bond_load* judged, uint8_t* judged_has, double* phi, int32_t* broken,
                 int32_t broken_cap, int32_t* retired, int32_t retired_cap, svxg_cascade_result* res) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!res || (P.n > 0 && (!f || !u)) || ((judged == nullptr) != (judged_has == nullptr)) || broken_cap < 0 ||
      retired_cap < 0) {
    set_error("svxg_cascade: bad arguments");
    return SVXG_ERR_ARG;
  }
  std::memset(res, 0, sizeof(*res));
  if (!P.have_graph) {
    set_error("svxg_cascade: no graph");
    return SVXG_ERR_STATE;
  }
  const svxg_cascade_options o = co ? *co : svxg_default_cascade_options();
  const int32_t max_breaks = std::max(1, o.max_breaks_per_round);  // (as world.cpp:61 clamps it)
  DeviceScope ds(P.device);
  const svxg_stress_options base = opt ? *opt : P.opt;
  svxg_stress_options multigrid_opt = base;
  multigrid_opt.amg_min_nodes = 0;  // (a structure restarted on a rebuilt preconditioner: world.cpp:1030)
  CascadeScratch S;
  TRY(cascade_alloc(P, S, max_breaks));
  struct Free {
    CascadeScratch& s;
    ~Free() { cascade_free(s); }
  } free_scratch{S};
  const size_t m6 = 6 * size_t(P.n);
  cudaStream_t st = P.stream;
  if (m6) {
    SVXG_CUDA(cudaMemcpyAsync(S.f, f, m6 * sizeof(double), cudaMemcpyHostToDevice, st));
    SVXG_CUDA(cudaMemcpyAsync(S.u, u, m6 * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  if (P.nb > 0) {
    if (judged) {
      SVXG_CUDA(cudaMemcpyAsync(S.judged, judged, sizeof(svxg_bond_load) * size_t(P.nb), cudaMemcpyHostToDevice, st));
      SVXG_CUDA(cudaMemcpyAsync(S.has, judged_has, size_t(P.nb), cudaMemcpyHostToDevice, st));
    } else {
      SVXG_CUDA(cudaMemsetAsync(S.has, 0, size_t(P.nb), st));
    }
    SVXG_CUDA(cudaMemsetAsync(S.phi, 0, sizeof(double) * size_t(P.nb), st));
  }
  bool shock = o.shock != 0, multigrid = false;
  int32_t restarts = 0;
  std::vector<int32_t> hb, hr;
  CascadeState hs{};
  auto read_state = [&]() -> int {
    SVXG_CUDA(cudaMemcpyAsync(&hs, S.st, sizeof(hs), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    return SVXG_OK;
  };
  for (;;) {
    if (!P.assembled) {
      int32_t ok = 0;
      TRY(assemble_impl(P, multigrid ? &multigrid_opt : &base, &ok));
      if (!ok) {
        res->status = SVXG_CASCADE_SINGULAR;
        break;
      }
    }
    if (m6) SVXG_CUDA(cudaMemcpyAsync(S.u0, S.u, m6 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    svxg_pcg_result r{};
    TRY(solve_common(P, S.f, S.u, o.rtol, o.maxit, 1, &r));
    res->solves += 1;
    res->pcg_iters += r.iters;
    res->rel_res = r.rel_res;
    if (r.breakdown) {
      if (m6) SVXG_CUDA(cudaMemcpyAsync(S.u, S.u0, m6 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      res->status = SVXG_CASCADE_BREAKDOWN;
      break;
    }
    if (!r.converged) {
      // world.cpp:1070-1093: keep the iterate unless it diverged; rebuild a stale or block-Jacobi
      // preconditioner; a current one that diverged starts again from rest
      const bool rebuild = !(P.assembled && P.pc_current) || P.jacobi_only;
      const bool diverging = !(r.rel_res < 10.0);
      if (diverging && m6) SVXG_CUDA(cudaMemcpyAsync(S.u, S.u0, m6 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if (rebuild) {
        P.assembled = false;
        P.active = false;
        multigrid = true;
      } else if (diverging && m6) {
        SVXG_CUDA(cudaMemsetAsync(S.u, 0, m6 * sizeof(double), st));
      }
      ++restarts;
      ++res->restarts;
      if (restarts >= o.solve_restarts) {
        res->status = SVXG_CASCADE_ABANDONED;
        break;
      }
      continue;
    }
    restarts = 0;
    if (r.iters > o.rebuild_after && (!(P.assembled && P.pc_current) || P.jacobi_only)) {
      P.assembled = false;  // (world.cpp:1109: the next solve rebuilds it)
      P.active = false;
    }
    TRY(cascade_judge(P, S, o.fragility, o.dif, shock && o.dif != 1.0 ? 1 : 0, o.break_band, max_breaks, BreakRule{}));
    TRY(read_state());
    {
      double mx = 0.0;
      std::memcpy(&mx, &hs.maxphi_bits, sizeof(mx));
      res->max_utilization = mx;
    }
    if (hs.m == 0) {
      res->status = SVXG_CASCADE_SETTLED;
      break;
    }
    if (res->rounds >= o.max_rounds) {
      res->status = SVXG_CASCADE_MAX_ROUNDS;
      break;
    }
    if (hs.K <= 0) {
      set_error("svxg_cascade: round selection failed");
      return SVXG_ERR_STATE;
    }
    const size_t old = hb.size();
    hb.resize(old + size_t(hs.K));
    SVXG_CUDA(cudaMemcpyAsync(hb.data() + old, S.sel, sizeof(int32_t) * size_t(hs.K), cudaMemcpyDeviceToHost, st));
    TRY(remove_bonds_list(P, S.sel, nullptr, hs.K, S.st));
    res->bonds_broken += hs.K;
    res->rounds += 1;
    shock = true;
    if (o.detach) {
      TRY(cascade_find_loose(P, S));
      TRY(read_state());
      if (hs.r > 0) {
        TRY(cascade_retire(P, S, hs.r));
        const size_t o2 = hr.size();
        hr.resize(o2 + size_t(hs.r));
        SVXG_CUDA(cudaMemcpyAsync(hr.data() + o2, S.nlist, sizeof(int32_t) * size_t(hs.r), cudaMemcpyDeviceToHost,
                                  st));
        res->nodes_retired += hs.r;
      }
    }
    TRY(read_state());
    if (P.assembled && !P.jacobi_only && (hs.any_in_k || hs.r_dof)) P.pc_current = false;
    P.active = false;
  }
  // results, and the host's copies of the flags the rounds changed
  if (m6) SVXG_CUDA(cudaMemcpyAsync(u, S.u, m6 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (P.nb > 0) {
    if (judged) {
      SVXG_CUDA(cudaMemcpyAsync(judged, S.judged, sizeof(svxg_bond_load) * size_t(P.nb), cudaMemcpyDeviceToHost, st));
      SVXG_CUDA(cudaMemcpyAsync(judged_has, S.has, size_t(P.nb), cudaMemcpyDeviceToHost, st));
    }
    if (phi) SVXG_CUDA(cudaMemcpyAsync(phi, S.phi, sizeof(double) * size_t(P.nb), cudaMemcpyDeviceToHost, st));
    TRY(cascade_bond_flags(P, S));
    P.h_broken.resize(size_t(P.nb));
    P.h_in_k.resize(size_t(P.nb));
    SVXG_CUDA(cudaMemcpyAsync(P.h_broken.data(), S.broken8, size_t(P.nb), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(cudaMemcpyAsync(P.h_in_k.data(), S.in_k8, size_t(P.nb), cudaMemcpyDeviceToHost, st));
  }
  SVXG_CUDA(host_wait(st));
  for (int32_t i : hr) P.h_nodes[size_t(i)].gone = 1;
  for (size_t k = 0; k < hb.size() && k < size_t(broken_cap); ++k) broken[k] = hb[k];
  for (size_t k = 0; k < hr.size() && k < size_t(retired_cap); ++k) retired[k] = hr[k];
  return SVXG_OK;
}


// SecAcc::finish + section_strengths(_general) (core/src/world/world_internal.hpp:130-441) on
// the device: host arrays in and out.
int svxg_build_bonds(const svxg_node* nodes, int32_t n, const svxg_section* secs, int32_t nb, const svxg_face* faces,
                     int64_t nf, const svxg_junction* juncs, int64_t nj, const svxg_lattice* lats, int32_t nl,
                     int32_t samples, const svxg_material* mats, svxg_bond* out) {
  if (n < 0 || nb < 0 || nf < 0 || nj < 0 || nl < 0 || samples < 1 ||
      (nb > 0 && (!nodes || !secs || !mats || !out)) || (nf > 0 && !faces) || (nj > 0 && !juncs) ||
      (nl > 0 && !lats)) {
    set_error("svxg_build_bonds: bad arguments");
    return SVXG_ERR_ARG;
  }
  for (int32_t k = 0; k < nb; ++k) {
    const svxg_section& S = secs[k];
    if (S.a < 0 || S.a >= n || S.b >= n || S.faces < 0 || S.first_face < 0 || S.first_face + S.faces > nf ||
        (S.b < 0 && S.axis > 2) || S.junctions < 0 ||
        (S.junctions > 0 && (S.first_junction < 0 || S.first_junction + S.junctions > nj)) ||
        (nl == 0 ? S.junctions != 0 : int32_t(S.grid) >= nl)) {
      set_error("svxg_build_bonds: section " + std::to_string(k) + " out of range");
      return SVXG_ERR_ARG;
    }
  }
  for (int64_t f = 0; f < nf; ++f)
    if (faces[f].axis > 2) {
      set_error("svxg_build_bonds: face axis out of range");
      return SVXG_ERR_ARG;
    }
  for (int64_t j = 0; j < nj; ++j)
    if (juncs[j].vg >= nl || juncs[j].face >= 6) {
      set_error("svxg_build_bonds: junction sample out of range");
      return SVXG_ERR_ARG;
    }
  if (nb == 0) return SVXG_OK;
  int dev = 0;
  SVXG_CUDA(cudaGetDevice(&dev));
  DeviceScope ds(dev);
  cudaStream_t st = cudaStreamPerThread;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t bn = up(sizeof(svxg_node) * size_t(std::max(n, 1))), bs = up(sizeof(svxg_section) * size_t(nb)),
               bf = up(sizeof(svxg_face) * size_t(std::max<int64_t>(nf, 1))),
               bj = up(sizeof(svxg_junction) * size_t(std::max<int64_t>(nj, 1))),
               bl = up(sizeof(svxg_lattice) * size_t(std::max(nl, 1))),
               bm = up(sizeof(svxg_material) * SVXG_MAX_MATERIALS), bo = up(sizeof(svxg_bond) * size_t(nb));
  char* base = nullptr;
  SVXG_CUDA(pool_malloc_async(reinterpret_cast<void**>(&base), bn + bs + bf + bj + bl + bm + bo + 256, st));
  char* c = base;
  svxg_node* dn = reinterpret_cast<svxg_node*>(c);
  c += bn;
  svxg_section* dsec = reinterpret_cast<svxg_section*>(c);
  c += bs;
  svxg_face* dfc = reinterpret_cast<svxg_face*>(c);
  c += bf;
  svxg_junction* djs = reinterpret_cast<svxg_junction*>(c);
  c += bj;
  svxg_lattice* dl = reinterpret_cast<svxg_lattice*>(c);
  c += bl;
  svxg_material* dm = reinterpret_cast<svxg_material*>(c);
  c += bm;
  svxg_bond* dout = reinterpret_cast<svxg_bond*>(c);
  c += bo;
  int32_t* dbad = reinterpret_cast<int32_t*>(c);
  int e = SVXG_OK;
  int32_t bad = 0;
  do {
    if (n > 0 && cudaMemcpyAsync(dn, nodes, sizeof(svxg_node) * size_t(n), cudaMemcpyHostToDevice, st)) break;
    if (cudaMemcpyAsync(dsec, secs, sizeof(svxg_section) * size_t(nb), cudaMemcpyHostToDevice, st)) break;
    if (nf > 0 && cudaMemcpyAsync(dfc, faces, sizeof(svxg_face) * size_t(nf), cudaMemcpyHostToDevice, st)) break;
    if (nj > 0 && cudaMemcpyAsync(djs, juncs, sizeof(svxg_junction) * size_t(nj), cudaMemcpyHostToDevice, st)) break;
    if (nl > 0 && cudaMemcpyAsync(dl, lats, sizeof(svxg_lattice) * size_t(nl), cudaMemcpyHostToDevice, st)) break;
    if (cudaMemcpyAsync(dm, mats, sizeof(svxg_material) * SVXG_MAX_MATERIALS, cudaMemcpyHostToDevice, st)) break;
    if (cudaMemsetAsync(dbad, 0, sizeof(int32_t), st)) break;
    e = build_bonds_device(dn, n, dsec, nb, dfc, nf, djs, nj, dl, nl, samples, dm, dout, dbad, st);
    if (e) break;
    if (cudaMemcpyAsync(out, dout, sizeof(svxg_bond) * size_t(nb), cudaMemcpyDeviceToHost, st)) break;
    if (cudaMemcpyAsync(&bad, dbad, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) break;
  } while (0);
  cudaError_t ce = cudaGetLastError();
  cudaFreeAsync(base, st);
  SVXG_CUDA(host_wait(st));
  if (e) return e;
  if (ce != cudaSuccess) {
    set_error(std::string("svxg_build_bonds: ") + cudaGetErrorString(ce));
    return SVXG_ERR_CUDA;
  }
  return bad ? SVXG_ERR_ARG : SVXG_OK;
}

int svxg_build_bonds_device(const svxg_node* nodes_dev, int32_t n, const svxg_section* secs_dev, int32_t nb,
                            const svxg_face* faces_dev, int64_t nf, const svxg_junction* juncs_dev, int64_t nj,
                            const svxg_lattice* lats_dev, int32_t nl, int32_t samples, const svxg_material* mats_dev,
                            svxg_bond* out_dev, int32_t* n_bad_dev, void* stream) {
  if (n < 0 || nb < 0 || nf < 0 || nj < 0 || nl < 0 || samples < 1 ||
      (nb > 0 && (!nodes_dev || !secs_dev || !mats_dev || !out_dev)) || (nf > 0 && !faces_dev) ||
      (nj > 0 && !juncs_dev) || (nl > 0 && !lats_dev)) {
    set_error("svxg_build_bonds_device: bad arguments");
    return SVXG_ERR_ARG;
  }
  return build_bonds_device(nodes_dev, n, secs_dev, nb, faces_dev, nf, juncs_dev, nj, lats_dev, nl, samples, mats_dev,
                            out_dev, n_bad_dev, static_cast<cudaStream_t>(stream));
}

// A loose piece's break rounds within one substep (World::Impl::body_stress_run,
// core/src/world/world_pieces.cpp:614-808). Per round the device solves, judges, picks and pays
// for the breaks and removes them; the host reads the round's counts and, when the piece splits
// from its pinned node, sorts its parts (their nodes are few) and moves the chips' loads.
int svxg_piece_rounds(svxg_problem* p, const svxg_stress_options* opt, const svxg_piece_options* po, const double* gf,
                      double* f, double* u, int32_t* broken, uint8_t* modes, int32_t broken_cap, int32_t* chips,
                      int32_t chips_cap, svxg_piece_result* res) {
  CHECK_P(p);
  Problem& P = p->P;
  if (!res || (P.n > 0 && (!f || !u)) || broken_cap < 0 || chips_cap < 0) {
    set_error("svxg_piece_rounds: bad arguments");
    return SVXG_ERR_ARG;
  }
  std::memset(res, 0, sizeof(*res));
  if (!P.have_graph) {
    set_error("svxg_piece_rounds: no graph");
    return SVXG_ERR_STATE;
  }
  const svxg_piece_options o = po ? *po : svxg_default_piece_options();
  const int32_t max_breaks = std::max(0, o.max_breaks_per_round);
  DeviceScope ds(P.device);
  svxg_stress_options so = opt ? *opt : P.opt;
  so.rtol = o.rtol;
  so.amg_min_nodes = 0;  // (small pieces: the coarsest level is the whole graph, solved exactly)
  CascadeScratch S;
  TRY(cascade_alloc(P, S, std::max(1, max_breaks)));
  struct Free {
    CascadeScratch& s;
    ~Free() { cascade_free(s); }
  } free_scratch{S};
  const int32_t n = P.n, nb = P.nb;
  const size_t m6 = 6 * size_t(n);
  cudaStream_t st = P.stream;
  std::vector<double> gfh(SVXG_MAX_MATERIALS, 2000.0);
  if (gf) std::copy(gf, gf + SVXG_MAX_MATERIALS, gfh.begin());
  SVXG_CUDA(cudaMemcpyAsync(S.gf, gfh.data(), sizeof(double) * SVXG_MAX_MATERIALS, cudaMemcpyHostToDevice, st));
  if (m6) {
    SVXG_CUDA(cudaMemcpyAsync(S.f, f, m6 * sizeof(double), cudaMemcpyHostToDevice, st));
    SVXG_CUDA(cudaMemcpyAsync(S.u, u, m6 * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  if (nb > 0) SVXG_CUDA(cudaMemsetAsync(S.phi, 0, sizeof(double) * size_t(nb), st));
  std::vector<int32_t> hb, hc;
  std::vector<uint8_t> hm;
  CascadeState hs{};
  auto read_state = [&]() -> int {
    SVXG_CUDA(cudaMemcpyAsync(&hs, S.st, sizeof(hs), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    return SVXG_OK;
  };
  double body_mass = 0.0;
  for (int32_t i = 0; i < n; ++i)
    if (!P.h_nodes[size_t(i)].gone) body_mass += P.h_nodes[size_t(i)].mass;
  BreakRule rule;
  rule.fraction = std::max(0.0, o.round_fraction);
  rule.energy = o.energy;
  rule.fracture_energy = o.fracture_energy;
  rule.crush_energy = o.crush_energy;
  rule.gf = S.gf;
  const bool impact = o.energy >= 0.0;
  const int32_t rounds = std::max(1, o.rounds);
  bool rebuilt = false;
  double spent = 0.0;
  if (!P.assembled) {
    int32_t ok = 0;
    TRY(assemble_impl(P, &so, &ok));
    if (!ok) {
      res->status = SVXG_PIECE_SINGULAR;
      return SVXG_OK;
    }
  }
  res->status = SVXG_PIECE_SETTLED;
  for (int32_t round = 0; round < rounds; ++round) {
    svxg_pcg_result r{};
    TRY(solve_common(P, S.f, S.u, o.rtol, o.maxit, 1, &r));
    const auto failed = [&](const svxg_pcg_result& x) {
      return !x.converged && (x.breakdown || x.rel_res > 5.0 * o.rtol);
    };
    if (failed(r) && round > 0 && !rebuilt) {
      // (the multigrid of the intact piece is stale after the breaks and the chips: rebuilt once)
      rebuilt = true;
      res->rebuilt = 1;
      P.assembled = false;
      P.active = false;
      int32_t ok = 0;
      TRY(assemble_impl(P, &so, &ok));
      if (ok) TRY(solve_common(P, S.f, S.u, o.rtol, o.maxit, 1, &r));
    }
    if (failed(r)) {
      P.assembled = false;
      P.active = false;
      if (m6) SVXG_CUDA(cudaMemsetAsync(S.u, 0, m6 * sizeof(double), st));
      res->status = SVXG_PIECE_SOLVE_FAILED;
      break;
    }
    res->checks += 1;
    res->pcg_iters += r.iters;
    rule.spent = spent;
    TRY(cascade_judge(P, S, o.fragility, 1.0, 0, o.break_band, std::max(1, max_breaks), rule));
    TRY(read_state());
    {
      double mx = 0.0;
      std::memcpy(&mx, &hs.maxphi_bits, sizeof(mx));
      if (round == 0) res->first_max_utilization = mx;
      res->max_utilization = mx;
    }
    if (hs.m == 0) {
      res->status = SVXG_PIECE_SETTLED;
      break;
    }
    // (max_breaks 0: the reference's loop takes none)
    const int32_t k = max_breaks == 0 ? 0 : hs.K;
    const bool poor = max_breaks == 0 ? false : hs.poor != 0;
    if (k < 0) {
      set_error("svxg_piece_rounds: round selection failed");
      return SVXG_ERR_STATE;
    }
    if (impact && max_breaks > 0) spent = hs.spent;
    if (k > 0) {
      const size_t old = hb.size();
      hb.resize(old + size_t(k));
      hm.resize(old + size_t(k));
      TRY(cascade_gather_modes(P, S, k));
      SVXG_CUDA(cudaMemcpyAsync(hb.data() + old, S.sel, sizeof(int32_t) * size_t(k), cudaMemcpyDeviceToHost, st));
      SVXG_CUDA(cudaMemcpyAsync(hm.data() + old, S.selmode, size_t(k), cudaMemcpyDeviceToHost, st));
      TRY(remove_bonds_list(P, S.sel, nullptr, k, S.st));
      res->bonds_broken += k;
    }
    res->spent = spent;
    if (poor || k == 0 || round + 1 == rounds) {
      res->status = poor ? SVXG_PIECE_ENERGY : (k == 0 ? SVXG_PIECE_SETTLED : SVXG_PIECE_LAST_ROUND);
      break;
    }
    int32_t pin = -1;
    for (int32_t i = 0; i < n; ++i)
      if (P.h_nodes[size_t(i)].fixed) pin = i;
    if (pin < 0) {
      res->status = SVXG_PIECE_NO_PIN;
      break;
    }
    // the parts: graph_components seeded by the pin (world_internal.hpp:660-705), component 0 the
    // pin's, the others numbered from 1 in node order (each root is its part's smallest node)
    TRY(cascade_roots(P, S));
    std::vector<int32_t> root(static_cast<size_t>(n));
    std::vector<uint8_t> brk(static_cast<size_t>(nb));
    SVXG_CUDA(cudaMemcpyAsync(root.data(), S.parent, sizeof(int32_t) * size_t(n), cudaMemcpyDeviceToHost, st));
    TRY(cascade_bond_flags(P, S));
    if (nb > 0) SVXG_CUDA(cudaMemcpyAsync(brk.data(), S.broken8, size_t(nb), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    std::vector<int32_t> comp(static_cast<size_t>(n), -1), number(static_cast<size_t>(n), -1);
    int32_t nc = 1;
    for (int32_t i = 0; i < n; ++i) {
      const int32_t rt = root[size_t(i)];
      if (rt == root[size_t(pin)]) {
        comp[size_t(i)] = 0;
      } else {
        if (number[size_t(rt)] < 0) number[size_t(rt)] = nc++;
        comp[size_t(i)] = number[size_t(rt)];
      }
    }
    if (nc <= 1) continue;
    std::vector<double> cmass(static_cast<size_t>(nc), 0.0);
    for (int32_t i = 0; i < n; ++i)
      if (!P.h_nodes[size_t(i)].gone) cmass[size_t(comp[size_t(i)])] += P.h_nodes[size_t(i)].mass;
    bool apart = false;
    for (int32_t c = 1; c < nc; ++c)
      if (cmass[size_t(c)] > o.chip_fraction * body_mass) apart = true;
    if (apart) {
      res->status = SVXG_PIECE_APART;
      break;
    }
    // chips pass their net load on to the nodes they broke from (world_pieces.cpp:752-797)
    std::vector<double> fh(m6);
    if (m6) SVXG_CUDA(cudaMemcpyAsync(fh.data(), S.f, m6 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(host_wait(st));
    std::vector<std::vector<int32_t>> attach(static_cast<size_t>(nc));
    for (int32_t b = 0; b < nb; ++b) {
      const int32_t ba = P.h_bond_ab[2 * size_t(b)], bb = P.h_bond_ab[2 * size_t(b) + 1];
      if (!brk[size_t(b)] || bb < 0) continue;
      const int32_t ca = comp[size_t(ba)], cb = comp[size_t(bb)];
      if (ca > 0 && cb == 0 && !P.h_nodes[size_t(bb)].gone) attach[size_t(ca)].push_back(bb);
      if (cb > 0 && ca == 0 && !P.h_nodes[size_t(ba)].gone) attach[size_t(cb)].push_back(ba);
    }
    auto cross = [](const double* a, const double* b, double* o3) {
      o3[0] = a[1] * b[2] - a[2] * b[1];
      o3[1] = a[2] * b[0] - a[0] * b[2];
      o3[2] = a[0] * b[1] - a[1] * b[0];
    };
    std::vector<double> cF(3 * size_t(nc), 0.0), cM(3 * size_t(nc), 0.0);
    std::vector<int32_t> chip_nodes;
    for (int32_t i = 0; i < n; ++i) {
      const int32_t c = comp[size_t(i)];
      if (c == 0 || P.h_nodes[size_t(i)].gone) continue;
      chip_nodes.push_back(i);
      auto& A = attach[size_t(c)];
      const svxg_v3& ci = P.h_nodes[size_t(i)].c;
      if (A.empty()) {
        double best = 1e300;
        int32_t bj = -1;
        for (int32_t j = 0; j < n; ++j) {
          if (comp[size_t(j)] != 0 || P.h_nodes[size_t(j)].gone) continue;
          const svxg_v3& cj = P.h_nodes[size_t(j)].c;
          const double dx = cj.x - ci.x, dy = cj.y - ci.y, dz = cj.z - ci.z;
          const double d = dx * dx + dy * dy + dz * dz;
          if (d < best) {
            best = d;
            bj = j;
          }
        }
        if (bj < 0) continue;
        A.push_back(bj);
      }
      double* fi = &fh[6 * size_t(i)];
      const double Fi[3] = {fi[0], fi[1], fi[2]};
      const double cc[3] = {ci.x, ci.y, ci.z};
      double t[3];
      cross(cc, Fi, t);
      for (int q = 0; q < 3; ++q) cF[3 * size_t(c) + q] += Fi[q];
      const double Mi[3] = {fi[3] + t[0], fi[4] + t[1], fi[5] + t[2]};
      for (int q = 0; q < 3; ++q) cM[3 * size_t(c) + q] += Mi[q];
      for (int q = 0; q < 6; ++q) fi[q] = 0.0;
    }
    for (int32_t c = 1; c < nc; ++c) {
      auto& A = attach[size_t(c)];
      if (A.empty()) continue;
      std::sort(A.begin(), A.end());
      A.erase(std::unique(A.begin(), A.end()), A.end());
      const double w = 1.0 / static_cast<double>(A.size());
      const double Fj[3] = {cF[3 * size_t(c)] * w, cF[3 * size_t(c) + 1] * w, cF[3 * size_t(c) + 2] * w};
      double Mr[3] = {cM[3 * size_t(c)], cM[3 * size_t(c) + 1], cM[3 * size_t(c) + 2]};
      for (int32_t j : A) {
        const svxg_v3& cj = P.h_nodes[size_t(j)].c;
        const double cc[3] = {cj.x, cj.y, cj.z};
        double t[3];
        cross(cc, Fj, t);
        for (int q = 0; q < 3; ++q) Mr[q] = Mr[q] - t[q];
      }
      const double Mj[3] = {Mr[0] * w, Mr[1] * w, Mr[2] * w};
      for (int32_t j : A) {
        double* fj = &fh[6 * size_t(j)];
        for (int q = 0; q < 3; ++q) {
          fj[q] += Fj[q];
          fj[3 + q] += Mj[q];
        }
      }
    }
    // (a chip holds together: its own bonds leave K but keep their topology)
    std::vector<int32_t> inner;
    for (int32_t b = 0; b < nb; ++b) {
      const int32_t ba = P.h_bond_ab[2 * size_t(b)], bb = P.h_bond_ab[2 * size_t(b) + 1];
      if (!brk[size_t(b)] && bb >= 0 && comp[size_t(ba)] > 0 && comp[size_t(ba)] == comp[size_t(bb)]) inner.push_back(b);
    }
    if (m6) SVXG_CUDA(cudaMemcpyAsync(S.f, fh.data(), m6 * sizeof(double), cudaMemcpyHostToDevice, st));
    const int32_t r_count = int32_t(chip_nodes.size());
    if (r_count > 0) {
      SVXG_CUDA(cudaMemcpyAsync(S.nlist, chip_nodes.data(), sizeof(int32_t) * size_t(r_count), cudaMemcpyHostToDevice,
                                st));
      SVXG_CUDA(cudaMemcpyAsync(&S.st->r, &r_count, sizeof(int32_t), cudaMemcpyHostToDevice, st));
      TRY(cascade_retire(P, S, r_count));
      if (!inner.empty()) {
        SVXG_CUDA(cudaMemcpyAsync(S.blist, inner.data(), sizeof(int32_t) * inner.size(), cudaMemcpyHostToDevice, st));
        TRY(unbreak_list(P, S.blist, int32_t(inner.size())));
      }
      for (int32_t i : chip_nodes) P.h_nodes[size_t(i)].gone = 1;
      hc.insert(hc.end(), chip_nodes.begin(), chip_nodes.end());
      res->chips += r_count;
    }
    TRY(read_state());
    if (P.assembled && !P.jacobi_only && (hs.any_in_k || hs.r_dof)) P.pc_current = false;
    P.active = false;
  }
  if (P.assembled && !P.jacobi_only && !hb.empty()) P.pc_current = false;
  if (m6) {
    SVXG_CUDA(cudaMemcpyAsync(u, S.u, m6 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(cudaMemcpyAsync(f, S.f, m6 * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  if (nb > 0) {
    TRY(cascade_bond_flags(P, S));
    P.h_broken.resize(size_t(nb));
    P.h_in_k.resize(size_t(nb));
    SVXG_CUDA(cudaMemcpyAsync(P.h_broken.data(), S.broken8, size_t(nb), cudaMemcpyDeviceToHost, st));
    SVXG_CUDA(cudaMemcpyAsync(P.h_in_k.data(), S.in_k8, size_t(nb), cudaMemcpyDeviceToHost, st));
  }
  SVXG_CUDA(host_wait(st));
  for (size_t t = 0; t < hb.size() && t < size_t(broken_cap); ++t) {
    if (broken) broken[t] = hb[t];
    if (modes) modes[t] = hm[t];
  }
  for (size_t t = 0; t < hc.size() && t < size_t(chips_cap); ++t)
    if (chips) chips[t] = hc[t];
  return SVXG_OK;
}

}  // extern "C"
