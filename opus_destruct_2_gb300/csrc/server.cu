// server.cu - the serving loop and the batched solve (include/svxg_server.h).
//
// Slots are host threads; each runs one request at a time on a problem of its own, so each
// request's kernels go to that problem's stream and requests overlap on the device (a solve's
// iterations are one graph launch, graphs.cu; allocations are stream-ordered from the library's
// pool and synchronize nothing else). One-shot requests use the slot's own problem, released
// after the result (its memory goes back to the pool for the next request); a structure kept
// resident owns its problem until it is evicted, and its problem object is then recycled.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "problem.cuh"
#include "svxg_server.h"

struct svxg_problem {
  svxg::Problem P;
};

namespace svxg {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  int64_t structure = -1;
  bool repeat = false;
  std::vector<svxg_node> nodes;
  std::vector<svxg_bond> bonds;
  std::vector<svxg_material> mats;
  std::vector<int32_t> remove;
  std::vector<double> f;
  int32_t n = 0;
  // a submission from device memory (svxg_server_submit_device / _repeat_device): the caller's
  // arrays are read when the request runs, in place of the host copies above
  const svxg_node* nodes_dev = nullptr;
  const svxg_bond* bonds_dev = nullptr;
  const svxg_material* mats_dev = nullptr;
  const double* f_dev = nullptr;
  int32_t nb_dev = 0;
  int32_t nbonds() const { return nodes_dev ? nb_dev : int32_t(bonds.size()); }
  const double* load() const { return f_dev ? f_dev : f.data(); }
  svxg_stress_options opt{};
  double rtol = 1e-6;
  int32_t maxit = -1;
  double fragility = 1.0;
  double* u_out = nullptr;
  int32_t* over_out = nullptr;
  Clock::time_point submitted;
  // a loose piece's break rounds instead of one solve and judgement (svxg_piece_rounds)
  bool piece = false;
  svxg_piece_options po{};
  std::vector<double> gf;
  std::vector<double> u0;
  double* f_out = nullptr;
  int32_t* broken_out = nullptr;
  uint8_t* modes_out = nullptr;
  int32_t* chips_out = nullptr;
  svxg_piece_result* piece_out = nullptr;
};

// New structures solved together as one problem (svxg_set_graphs) and kept for their repeats: the
// problem holds every member's K, the batch's multigrid and last solution; a repeat of a member
// removes its bonds in place (offset into the batch) and solves the batch warm with that member's
// new load. members[g]: graph g's structure id (-1: a one-shot request or a dropped structure).
struct Bundle {
  svxg_problem* p = nullptr;
  std::vector<int64_t> members;
  std::vector<int32_t> n, nb;
  std::vector<int64_t> node_off, bond_off;
  int32_t live = 0;
  int64_t bytes = 0;
};

struct Resident {
  svxg_problem* p = nullptr;
  int64_t bytes = 0;
  bool forget = false;
  std::list<int64_t>::iterator lru;
  std::shared_ptr<Bundle> bundle;  // (a member of a batch: p is the bundle's problem, bytes 0)
  int32_t member = -1;
};

// A new structure's device bytes before it exists, from its sizes: K (one diagonal block per
// node and two per bond, FP64 and FP32), the multigrid hierarchy (about K again), the run and
// cycle vectors and the graph itself, with a margin.
int64_t estimate_bytes(int64_t n, int64_t nb) {
  const int64_t blocks = n + 2 * nb;
  return blocks * 36 * 12 * 2 + n * 6 * 8 * 24 + n * 40 + nb * 216 + (int64_t(1) << 20);
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int d) {
    cudaGetDevice(&prev);
    cudaSetDevice(d);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// A slot's CUDA stream and pinned scalar mirrors, lent to whichever problem the slot runs (so a
// resident structure holds device memory only, not a stream or pinned host memory of its own).
struct Slot {
  cudaStream_t stream = nullptr;
  void* h_s = nullptr;
  void* h_ms = nullptr;
  int init() {
    SVXG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    SVXG_CUDA(cudaMallocHost(&h_s, 256));
    SVXG_CUDA(cudaMallocHost(&h_ms, 256));
    return SVXG_OK;
  }
  ~Slot() {
    if (stream) cudaStreamSynchronize(stream);
    if (h_s) cudaFreeHost(h_s);
    if (h_ms) cudaFreeHost(h_ms);
    if (stream) cudaStreamDestroy(stream);
  }
  void lend(svxg_problem* p) const {
    Problem& P = p->P;
    P.stream = stream;
    P.mem.stream = stream;
    P.h_s = static_cast<PcgScalars*>(h_s);
    P.h_ms = h_ms;
  }
};

// a problem without a stream or pinned mirrors of its own (a slot lends them)
int create_bare(svxg_problem** out, int device) {
  *out = nullptr;
  svxg_problem* p = new (std::nothrow) svxg_problem;
  if (!p) return SVXG_ERR_NOMEM;
  p->P.device = device;
  p->P.borrowed = true;
  p->P.opt = svxg_default_options();
  *out = p;
  return SVXG_OK;
}

}  // namespace
}  // namespace svxg

using namespace svxg;

struct svxg_server {
  int device = 0;
  int64_t budget = 0;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_mem;
  std::deque<Request> queue;
  bool stop = false;
  int64_t outstanding = 0;
  std::unordered_map<int64_t, Resident> resident;
  std::list<int64_t> lru;                // front: least recently used
  std::unordered_set<int64_t> running_structures;
  std::unordered_map<int64_t, std::vector<Request>> deferred;
  std::vector<svxg_problem*> spare;      // problem objects of evicted structures
  int64_t resident_bytes = 0;
  int64_t running_bytes = 0;             // estimates of the requests running
  int64_t next_ticket = 1;
  std::unordered_map<int64_t, svxg_request_result> done;
  std::vector<double> latencies;
  int64_t completed = 0, failed = 0, evictions = 0, admission_waits = 0, peak = 0;
  Clock::time_point t_first{}, t_last{};
  bool any = false;
  bool blocking = false;
  Slot admin;  // (lent to problems released outside a slot: forget, destroy)
  // batching of new requests (svxg_server_set_batching): at most batch_graphs graphs of at most
  // batch_graph_nodes nodes each and batch_nodes in all go into one problem
  int32_t batch_graphs = 16;
  int32_t batch_graph_nodes = 20000;
  int64_t batch_nodes = 65536;
  int64_t batches = 0, batched_requests = 0;
  bool hold = false;  // (svxg_server_hold: slots take no new work)
};

namespace {

// a bundle released (all its members gone): its problem back to the spares
void release_bundle_locked(svxg_server* S, Bundle& b, const Slot& slot) {
  if (!b.p) return;
  slot.lend(b.p);
  svxg_release(b.p);
  S->spare.push_back(b.p);
  S->resident_bytes -= b.bytes;
  b.p = nullptr;
  b.bytes = 0;
}

// resident structure `it` no longer kept (evicted, forgotten, replaced or failed): a single
// problem goes back to the spares; a bundle member is dropped, and the bundle with its last member
void drop_resident_locked(svxg_server* S, std::unordered_map<int64_t, Resident>::iterator it, const Slot& slot) {
  Resident& r = it->second;
  if (r.bundle) {
    Bundle& b = *r.bundle;
    if (r.member >= 0 && r.member < int32_t(b.members.size()) && b.members[size_t(r.member)] == it->first) {
      b.members[size_t(r.member)] = -1;
      --b.live;
    }
    if (b.live <= 0) release_bundle_locked(S, b, slot);
  } else {
    slot.lend(r.p);
    svxg_release(r.p);
    S->spare.push_back(r.p);
    S->resident_bytes -= r.bytes;
  }
  S->lru.erase(r.lru);
  S->resident.erase(it);
}

bool bundle_running_locked(const svxg_server* S, const Bundle& b) {
  for (int64_t m : b.members)
    if (m >= 0 && S->running_structures.count(m)) return true;
  return false;
}

void evict_locked(svxg_server* S, int64_t need, const Slot& slot) {
  for (auto it = S->lru.begin(); it != S->lru.end() && S->resident_bytes + S->running_bytes + need > S->budget;) {
    auto r = S->resident.find(*it);
    if (r == S->resident.end() || S->running_structures.count(*it)) {
      ++it;
      continue;
    }
    if (r->second.bundle) {
      // (a bundle frees memory only as a whole: every member goes, unless one is running)
      std::shared_ptr<Bundle> b = r->second.bundle;
      if (bundle_running_locked(S, *b)) {
        ++it;
        continue;
      }
      for (int64_t m : std::vector<int64_t>(b->members)) {
        auto q = S->resident.find(m);
        if (m >= 0 && q != S->resident.end() && q->second.bundle == b) {
          drop_resident_locked(S, q, slot);
          ++S->evictions;
        }
      }
      it = S->lru.begin();
      continue;
    }
    ++it;
    drop_resident_locked(S, r, slot);
    ++S->evictions;
  }
}

void record(svxg_server* S, const Request& q, svxg_request_result res) {
  const auto t = Clock::now();
  res.ticket = q.ticket;
  res.latency_ms = std::chrono::duration<double, std::milli>(t - q.submitted).count();
  std::lock_guard<std::mutex> lk(S->mu);
  S->done[q.ticket] = res;
  S->latencies.push_back(res.latency_ms);
  if (res.status == SVXG_OK) ++S->completed;
  else ++S->failed;
  S->t_last = t;
  --S->outstanding;
  S->cv_done.notify_all();
}

int judge_into(svxg_problem* p, const Request& q, svxg_request_result* res) {
  int32_t nover = 0;
  const int32_t cap = q.over_out ? p->P.nb : 0;
  const int e = svxg_utilization(p, q.fragility, nullptr, nullptr, q.over_out, cap, &nover);
  res->failing = nover;
  return e;
}

int run_piece(svxg_problem* p, Request& q, svxg_request_result* res) {
  std::vector<double> u(6 * size_t(q.n), 0.0);
  if (!q.u0.empty()) u = q.u0;
  svxg_piece_result pr{};
  const int32_t nb = int32_t(q.bonds.size());
  const int e = svxg_piece_rounds(p, &q.opt, &q.po, q.gf.data(), q.f.data(), u.data(), q.broken_out, q.modes_out,
                                  q.broken_out || q.modes_out ? nb : 0, q.chips_out, q.chips_out ? q.n : 0, &pr);
  if (e) return e;
  if (q.u_out) std::copy(u.begin(), u.end(), q.u_out);
  if (q.f_out) std::copy(q.f.begin(), q.f.end(), q.f_out);
  if (q.piece_out) *q.piece_out = pr;
  res->iters = pr.pcg_iters;
  res->converged = pr.status != SVXG_PIECE_SOLVE_FAILED && pr.status != SVXG_PIECE_SINGULAR;
  res->breakdown = pr.status == SVXG_PIECE_SINGULAR;
  res->failing = pr.bonds_broken;
  res->rel_res = 0.0;
  return SVXG_OK;
}

int run_new(svxg_problem* p, Request& q, svxg_request_result* res) {
  int e = q.nodes_dev ? svxg_set_graph_device(p, q.nodes_dev, q.n, q.bonds_dev, q.nb_dev, q.mats_dev)
                      : svxg_set_graph(p, q.nodes.data(), q.n, q.bonds.data(), int32_t(q.bonds.size()), q.mats.data());
  if (e) return e;
  if (q.piece) return run_piece(p, q, res);
  int32_t ok = 0;
  e = svxg_assemble(p, &q.opt, &ok);
  if (e) return e;
  if (!ok) {
    res->breakdown = 1;
    res->rel_res = INFINITY;
    return SVXG_OK;
  }
  std::vector<double> u;
  double* uo = q.u_out;
  if (!uo) {
    u.resize(6 * size_t(q.n));
    uo = u.data();
  }
  svxg_pcg_result r{};
  e = solve_nodes_host(p->P, q.load(), uo, q.rtol, q.maxit, kCold, &r);
  if (e) return e;
  res->iters = r.iters;
  res->converged = r.converged;
  res->breakdown = r.breakdown;
  res->rel_res = r.rel_res;
  res->err_est = p->P.last_err_est;
  return judge_into(p, q, res);
}

int run_repeat(svxg_problem* p, Request& q, svxg_request_result* res) {
  if (q.n != p->P.n) {
    set_error("repeat request: node count differs from the resident structure's");
    return SVXG_ERR_ARG;
  }
  if (!q.remove.empty()) {
    const int e = svxg_remove_bonds(p, q.remove.data(), int32_t(q.remove.size()));
    if (e) return e;
  }
  svxg_pcg_result r{};
  const int e = solve_nodes_host(p->P, q.load(), q.u_out, q.rtol, q.maxit, kWarmResident, &r);
  if (e) return e;
  res->warm = 1;
  res->iters = r.iters;
  res->converged = r.converged;
  res->breakdown = r.breakdown;
  res->rel_res = r.rel_res;
  res->err_est = p->P.last_err_est;
  return judge_into(p, q, res);
}

// ---- batches -------------------------------------------------------------------------------

bool same_options(const Request& a, const Request& b) {
  if ((a.nodes_dev != nullptr) != (b.nodes_dev != nullptr)) return false;
  if (a.rtol != b.rtol || a.maxit != b.maxit || a.fragility != b.fragility) return false;
  if (std::memcmp(&a.opt, &b.opt, sizeof(a.opt)) != 0) return false;
  if (a.nodes_dev) return a.mats_dev == b.mats_dev;
  return a.mats.size() == b.mats.size() &&
         std::memcmp(a.mats.data(), b.mats.data(), sizeof(svxg_material) * a.mats.size()) == 0;
}

bool batchable(const svxg_server* S, const Request& q) {
  return S->batch_graphs > 1 && !q.repeat && !q.piece && q.n > 0 && q.n <= S->batch_graph_nodes;
}

// the failing bonds of graph g of a batch from the batch's ascending list (its own numbering)
int32_t member_failures(const std::vector<int32_t>& over, int32_t n_over, int64_t b0, int64_t b1, int32_t* out) {
  const auto first = std::lower_bound(over.begin(), over.begin() + n_over, int32_t(b0));
  const auto last = std::lower_bound(first, over.begin() + n_over, int32_t(b1));
  int32_t k = 0;
  for (auto it = first; it != last; ++it, ++k)
    if (out) out[k] = int32_t(*it - b0);
  return k;
}

// New requests as one problem: graphs one after another, assembled and solved together (every
// launch over the whole batch, each graph stopping at its own target), judged, and each request's
// result (its u, failure list and count, rel. residual) taken out of the batch's.
int run_batch(svxg_problem* p, std::vector<Request>& B, std::vector<svxg_request_result>& res, Bundle& shape) {
  const int32_t count = int32_t(B.size());
  const size_t cnt = static_cast<size_t>(count);
  const bool dev = B[0].nodes_dev != nullptr;
  std::vector<const svxg_node*> np(cnt);
  std::vector<const svxg_bond*> bp(cnt);
  std::vector<const double*> fp(cnt);
  std::vector<double*> up(cnt);
  std::vector<int32_t> n(cnt), nb(cnt);
  for (size_t g = 0; g < cnt; ++g) {
    const Request& q = B[g];
    np[g] = dev ? q.nodes_dev : q.nodes.data();
    bp[g] = dev ? q.bonds_dev : q.bonds.data();
    fp[g] = q.load();
    up[g] = q.u_out;
    n[g] = q.n;
    nb[g] = q.nbonds();
  }
  int e = dev ? svxg_set_graphs_device(p, count, np.data(), n.data(), bp.data(), nb.data(), B[0].mats_dev)
              : svxg_set_graphs(p, count, np.data(), n.data(), bp.data(), nb.data(), B[0].mats.data());
  if (e) return e;
  shape.n = n;
  shape.nb = nb;
  shape.node_off = p->P.seg_node;
  shape.bond_off = p->P.seg_bond;
  int32_t ok = 0;
  e = svxg_assemble(p, &B[0].opt, &ok);
  if (e) return e;
  if (!ok) {
    for (auto& r : res) {
      r.breakdown = 1;
      r.rel_res = INFINITY;
    }
    return SVXG_OK;
  }
  svxg_pcg_result pr{};
  e = batch_solve_loads(p->P, fp.data(), nullptr, up.data(), B[0].rtol, B[0].maxit, false, &pr);
  if (e) return e;
  std::vector<double> rel(cnt, 0.0);
  std::vector<int32_t> conv(cnt, 0), iters(cnt, 0);
  std::vector<double> est(cnt, 0.0);
  e = svxg_graph_results(p, count, rel.data(), conv.data(), iters.data(), est.data());
  if (e) return e;
  std::vector<int32_t> over(size_t(std::max(p->P.nb, 1)));
  int32_t n_over = 0;
  e = svxg_utilization(p, B[0].fragility, nullptr, nullptr, over.data(), int32_t(over.size()), &n_over);
  if (e) return e;
  for (size_t g = 0; g < cnt; ++g) {
    svxg_request_result& r = res[g];
    r.iters = iters[g];
    r.err_est = est[g];
    r.breakdown = pr.breakdown;
    r.converged = conv[g] && !pr.breakdown;
    r.rel_res = pr.breakdown && !std::isfinite(pr.rel_res) ? INFINITY : rel[g];
    r.failing = member_failures(over, n_over, shape.bond_off[g], shape.bond_off[g + 1], B[g].over_out);
  }
  return SVXG_OK;
}

// Repeats of members of one bundle (distinct members; member[i] is R[i]'s): every member's removals
// in one in-place pass (offset into the batch), their new loads over theirs, the batch solved warm
// from its last solution (members without a repeat start at their converged state), each request's
// result.
int run_bundle_repeats(Bundle& b, std::vector<Request>& R, const std::vector<int32_t>& member,
                       std::vector<svxg_request_result>& res) {
  svxg_problem* p = b.p;
  const size_t count = b.members.size();
  std::vector<int32_t> rm;
  std::vector<const double*> fp(count, nullptr);
  std::vector<double*> up(count, nullptr);
  std::vector<uint8_t> take(count, 0);
  for (size_t i = 0; i < R.size(); ++i) {
    const size_t g = size_t(member[i]);
    const Request& q = R[i];
    if (q.n != b.n[g]) {
      set_error("repeat request: node count differs from the resident structure's");
      return SVXG_ERR_ARG;
    }
    for (int32_t k : q.remove) {
      if (k < 0 || k >= b.nb[g]) {
        set_error("repeat request: bond index out of range");
        return SVXG_ERR_ARG;
      }
      rm.push_back(int32_t(b.bond_off[g] + k));
    }
    fp[g] = q.load();
    up[g] = q.u_out;
    take[g] = 1;
  }
  if (!rm.empty()) {
    const int e = svxg_remove_bonds(p, rm.data(), int32_t(rm.size()));
    if (e) return e;
  }
  svxg_pcg_result pr{};
  int e = batch_solve_loads(p->P, fp.data(), take.data(), up.data(), R[0].rtol, R[0].maxit, true, &pr);
  if (e) return e;
  std::vector<double> rel(count, 0.0);
  std::vector<int32_t> conv(count, 0), iters(count, 0);
  std::vector<double> est(count, 0.0);
  e = svxg_graph_results(p, int32_t(count), rel.data(), conv.data(), iters.data(), est.data());
  if (e) return e;
  std::vector<int32_t> over(size_t(std::max(p->P.nb, 1)));
  int32_t n_over = 0;
  e = svxg_utilization(p, R[0].fragility, nullptr, nullptr, over.data(), int32_t(over.size()), &n_over);
  if (e) return e;
  for (size_t i = 0; i < R.size(); ++i) {
    const size_t g = size_t(member[i]);
    svxg_request_result& r = res[i];
    r.warm = 1;
    r.iters = iters[g];
    r.err_est = est[g];
    r.breakdown = pr.breakdown;
    r.converged = conv[g] && !pr.breakdown;
    r.rel_res = pr.breakdown && !std::isfinite(pr.rel_res) ? INFINITY : rel[g];
    r.failing = member_failures(over, n_over, b.bond_off[g], b.bond_off[g + 1], R[i].over_out);
  }
  return SVXG_OK;
}

// the structure ids a piece of work runs under (every live member of a bundle it uses)
void mark_running_locked(svxg_server* S, const std::vector<int64_t>& ids) {
  for (int64_t id : ids)
    if (id >= 0) S->running_structures.insert(id);
}

// ... and their release: requests parked behind them go back to the head of the queue
void unmark_running_locked(svxg_server* S, const std::vector<int64_t>& ids) {
  bool requeued = false;
  for (int64_t id : ids) {
    if (id < 0) continue;
    S->running_structures.erase(id);
    auto d = S->deferred.find(id);
    if (d != S->deferred.end()) {
      for (auto it = d->second.rbegin(); it != d->second.rend(); ++it) S->queue.push_front(std::move(*it));
      S->deferred.erase(d);
      requeued = true;
    }
  }
  if (requeued) S->cv_work.notify_all();
}

// ---- the slots ------------------------------------------------------------------------------
// A request for structure s waits while another request for s runs (or for any member of s's
// bundle): it parks in deferred[s] and goes back to the head of the queue when that one finishes.
// (A repeat submitted after its structure's first request therefore always finds it resident,
// unless it was evicted.)

constexpr size_t kBatchScan = 512;  // queued requests a slot looks through to fill a batch

void worker(svxg_server* S) {
  cudaSetDevice(S->device);
  Slot slot;
  const int slot_ok = slot.init();
  svxg_problem* own = nullptr;
  for (;;) {
    Request q;
    std::vector<Request> group;        // the requests run with q: a batch of new ones, or repeats on one bundle
    std::vector<int32_t> gmember;      // (repeats on a bundle: each one's member, q's first)
    std::shared_ptr<Bundle> bundle;
    std::vector<int64_t> locks;        // structure ids held while this runs
    svxg_problem* p = nullptr;
    int64_t est = 0;
    bool keep = false, admitted = false;
    int e = SVXG_OK;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        S->cv_work.wait(lk, [&] { return S->stop || (!S->queue.empty() && !S->hold); });
        if (S->queue.empty()) break;
        // (taken into its own variable: a deferred request leaves q as it was - ticket 0 - so a
        // stop that finds the queue empty afterwards runs nothing)
        Request r = std::move(S->queue.front());
        S->queue.pop_front();
        if (r.structure >= 0 && S->running_structures.count(r.structure)) {
          S->deferred[r.structure].push_back(std::move(r));
          continue;
        }
        q = std::move(r);
        break;
      }
      if (q.ticket == 0) break;  // (stopped, nothing left)
      if (q.repeat) {
        auto it = S->resident.find(q.structure);
        if (it == S->resident.end()) {
          set_error("repeat request: the structure is not resident");
          e = SVXG_ERR_STATE;
          locks.push_back(q.structure);
        } else if (it->second.bundle) {
          // repeats of other members of the same bundle queued behind it join this solve
          bundle = it->second.bundle;
          gmember.push_back(it->second.member);
          std::vector<uint8_t> taken(bundle->members.size(), 0);
          taken[size_t(it->second.member)] = 1;
          std::vector<Request> rest;
          for (size_t scanned = 0; scanned < kBatchScan && !S->queue.empty(); ++scanned) {
            Request r = std::move(S->queue.front());
            S->queue.pop_front();
            auto jt = r.repeat ? S->resident.find(r.structure) : S->resident.end();
            if (jt != S->resident.end() && jt->second.bundle == bundle && !taken[size_t(jt->second.member)] &&
                r.rtol == q.rtol && r.maxit == q.maxit && r.fragility == q.fragility) {
              taken[size_t(jt->second.member)] = 1;
              gmember.push_back(jt->second.member);
              group.push_back(std::move(r));
            } else {
              rest.push_back(std::move(r));
            }
          }
          for (auto rt = rest.rbegin(); rt != rest.rend(); ++rt) S->queue.push_front(std::move(*rt));
          for (int64_t m : bundle->members)
            if (m >= 0) {
              locks.push_back(m);
              auto mt = S->resident.find(m);
              if (mt != S->resident.end()) {
                S->lru.erase(mt->second.lru);
                mt->second.lru = S->lru.insert(S->lru.end(), m);
              }
            }
          p = bundle->p;
        } else {
          p = it->second.p;
          S->lru.erase(it->second.lru);
          it->second.lru = S->lru.insert(S->lru.end(), q.structure);
          locks.push_back(q.structure);
        }
      } else {
        locks.push_back(q.structure);
        est = estimate_bytes(q.n, int64_t(q.nbonds()));
        if (batchable(S, q)) {
          // further new requests with the same options join it as one problem
          int64_t nodes = q.n;
          std::unordered_set<int64_t> ids;
          if (q.structure >= 0) ids.insert(q.structure);
          std::vector<Request> rest;
          for (size_t scanned = 0;
               scanned < kBatchScan && !S->queue.empty() && int32_t(group.size()) + 1 < S->batch_graphs; ++scanned) {
            Request r = std::move(S->queue.front());
            S->queue.pop_front();
            const bool fits = batchable(S, r) && nodes + r.n <= S->batch_nodes && same_options(q, r) &&
                              (r.structure < 0 || (!ids.count(r.structure) && !S->running_structures.count(r.structure)));
            if (fits) {
              nodes += r.n;
              if (r.structure >= 0) ids.insert(r.structure);
              locks.push_back(r.structure);
              est += estimate_bytes(r.n, int64_t(r.nbonds()));
              group.push_back(std::move(r));
            } else {
              rest.push_back(std::move(r));
            }
          }
          for (auto rt = rest.rbegin(); rt != rest.rend(); ++rt) S->queue.push_front(std::move(*rt));
        }
        if (est > S->budget) {
          set_error("request exceeds the server's HBM budget");
          e = SVXG_ERR_NOMEM;
        } else {
          evict_locked(S, est, slot);
          if (S->resident_bytes + S->running_bytes + est > S->budget) {
            ++S->admission_waits;
            S->cv_mem.wait(lk, [&] {
              evict_locked(S, est, slot);
              return S->resident_bytes + S->running_bytes + est <= S->budget;
            });
          }
          S->running_bytes += est;
          admitted = true;
          S->peak = std::max(S->peak, S->resident_bytes + S->running_bytes);
          keep = q.structure >= 0;
          for (const Request& r : group) keep = keep || r.structure >= 0;
          // (resubmitted structures: the new graph replaces the old)
          for (int64_t id : locks) {
            auto old = id >= 0 ? S->resident.find(id) : S->resident.end();
            if (old != S->resident.end()) drop_resident_locked(S, old, slot);
          }
          if (keep && !S->spare.empty()) {
            p = S->spare.back();
            S->spare.pop_back();
          }
        }
      }
      mark_running_locked(S, locks);
    }
    // ---- run ----
    const bool batch = !q.repeat && !group.empty();
    group.insert(group.begin(), std::move(q));
    std::vector<svxg_request_result> res(group.size());
    const auto taken_at = Clock::now();
    for (size_t i = 0; i < group.size(); ++i)
      res[i].queue_ms = std::chrono::duration<double, std::milli>(taken_at - group[i].submitted).count();
    if (!e && slot_ok) e = slot_ok;
    if (!e && !p && !keep) {
      if (!own) e = create_bare(&own, S->device);
      p = own;
    } else if (!e && !p) {
      e = create_bare(&p, S->device);
    }
    Bundle shape;
    if (!e) {
      slot.lend(p);
      if (bundle) {
        e = run_bundle_repeats(*bundle, group, gmember, res);
      } else if (batch) {
        e = run_batch(p, group, res, shape);
      } else {
        e = group[0].repeat ? run_repeat(p, group[0], &res[0]) : run_new(p, group[0], &res[0]);
      }
    }
    for (auto& r : res) r.status = e;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      if (admitted) S->running_bytes -= est;
      if (bundle) {
        const int64_t bb = bundle->p ? bundle->p->P.mem.bytes : 0;
        S->resident_bytes += bb - bundle->bytes;
        bundle->bytes = bb;
        for (int64_t m : std::vector<int64_t>(bundle->members)) {
          auto mt = m >= 0 ? S->resident.find(m) : S->resident.end();
          // (a failed repeat: the whole bundle is dropped, its state unknown)
          if (mt != S->resident.end() && (e || mt->second.forget)) drop_resident_locked(S, mt, slot);
        }
      } else if (group[0].repeat) {
        auto it = S->resident.find(group[0].structure);
        if (it != S->resident.end()) {
          const int64_t b = it->second.p->P.mem.bytes;
          S->resident_bytes += b - it->second.bytes;
          it->second.bytes = b;
          if (it->second.forget || e) drop_resident_locked(S, it, slot);  // (a failed repeat: dropped)
        }
      } else if (keep && p) {
        if (!e && batch) {
          auto b = std::make_shared<Bundle>(std::move(shape));
          b->p = p;
          b->bytes = p->P.mem.bytes;
          b->members.assign(group.size(), -1);
          for (size_t g = 0; g < group.size(); ++g) {
            const int64_t id = group[g].structure;
            if (id < 0) continue;
            b->members[g] = id;
            ++b->live;
            Resident r;
            r.p = p;
            r.bundle = b;
            r.member = int32_t(g);
            r.lru = S->lru.insert(S->lru.end(), id);
            S->resident[id] = r;
          }
          S->resident_bytes += b->bytes;
        } else if (!e) {
          Resident r;
          r.p = p;
          r.bytes = p->P.mem.bytes;
          r.lru = S->lru.insert(S->lru.end(), group[0].structure);
          S->resident[group[0].structure] = r;
          S->resident_bytes += r.bytes;
        } else {
          svxg_release(p);
          S->spare.push_back(p);
        }
      } else if (p && p == own) {
        svxg_release(own);
      }
      if (batch) {
        ++S->batches;
        S->batched_requests += int64_t(group.size());
      }
      S->peak = std::max(S->peak, S->resident_bytes + S->running_bytes);
      unmark_running_locked(S, locks);
      S->cv_mem.notify_all();
    }
    for (size_t i = 0; i < group.size(); ++i) record(S, group[i], res[i]);
    pool_trim(size_t(1) << 30);  // (this slot's pool keeps at most 1 GiB it is not using)
  }
  if (own) svxg_problem_destroy(own);
}

int64_t submit(svxg_server* S, Request&& q) {
  q.submitted = Clock::now();
  int64_t t;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return SVXG_ERR_STATE;
    t = q.ticket = S->next_ticket++;
    if (!S->any) {
      S->t_first = q.submitted;
      S->any = true;
    }
    ++S->outstanding;
    S->queue.push_back(std::move(q));
  }
  S->cv_work.notify_one();
  return t;
}

}  // namespace

extern "C" {

int svxg_server_create(svxg_server** out, int device, int64_t hbm_budget_bytes, int32_t workers) {
  if (!out || workers <= 0 || workers > 256 || hbm_budget_bytes <= 0) {
    set_error("svxg_server_create: bad arguments");
    return SVXG_ERR_ARG;
  }
  *out = nullptr;
  if (device < 0 || svxg_device_count() <= device) {
    set_error("no such CUDA device");
    return SVXG_ERR_NODEVICE;
  }
  svxg_server* S = new svxg_server;
  S->device = device;
  S->budget = hbm_budget_bytes;
  {
    DeviceGuard g(device);
    const int e = S->admin.init();
    if (e) {
      delete S;
      return e;
    }
  }
  S->blocking = workers > 1;
  if (S->blocking) blocking_waits(true);
  for (int32_t i = 0; i < workers; ++i) S->threads.emplace_back(worker, S);
  *out = S;
  return SVXG_OK;
}

void svxg_server_destroy(svxg_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->threads) t.join();
  // (the members of a bundle share its problem: each problem is destroyed once)
  std::unordered_set<svxg_problem*> gone;
  for (auto& kv : S->resident) {
    if (!kv.second.p || !gone.insert(kv.second.p).second) continue;
    S->admin.lend(kv.second.p);
    svxg_problem_destroy(kv.second.p);
  }
  for (svxg_problem* p : S->spare) {
    S->admin.lend(p);
    svxg_problem_destroy(p);
  }
  if (S->blocking) blocking_waits(false);
  delete S;
}

int64_t svxg_server_submit(svxg_server* S, int64_t structure, const svxg_node* nodes, int32_t n,
                           const svxg_bond* bonds, int32_t nb, const svxg_material* mats, const double* f,
                           const svxg_stress_options* opt, double rtol, int32_t maxit, double fragility,
                           double* u_out, int32_t* over_out) {
  if (!S || n < 0 || nb < 0 || !mats || (n > 0 && (!nodes || !f)) || (nb > 0 && !bonds)) {
    set_error("svxg_server_submit: bad arguments");
    return SVXG_ERR_ARG;
  }
  Request q;
  q.structure = structure;
  q.n = n;
  q.nodes.assign(nodes, nodes + n);
  q.bonds.assign(bonds, bonds + nb);
  q.mats.assign(mats, mats + SVXG_MAX_MATERIALS);
  q.f.assign(f, f + 6 * size_t(n));
  q.opt = opt ? *opt : svxg_default_options();
  q.rtol = rtol;
  q.maxit = maxit;
  q.fragility = fragility;
  q.u_out = u_out;
  q.over_out = over_out;
  return submit(S, std::move(q));
}

int64_t svxg_server_submit_repeat(svxg_server* S, int64_t structure, const int32_t* remove, int32_t nremove,
                                  const double* f, int32_t n, double rtol, int32_t maxit, double fragility,
                                  double* u_out, int32_t* over_out) {
  if (!S || structure < 0 || nremove < 0 || (nremove > 0 && !remove) || n < 0 || (n > 0 && !f)) {
    set_error("svxg_server_submit_repeat: bad arguments");
    return SVXG_ERR_ARG;
  }
  Request q;
  q.structure = structure;
  q.repeat = true;
  q.n = n;
  q.remove.assign(remove, remove + nremove);
  q.f.assign(f, f + 6 * size_t(n));
  q.rtol = rtol;
  q.maxit = maxit;
  q.fragility = fragility;
  q.u_out = u_out;
  q.over_out = over_out;
  return submit(S, std::move(q));
}

int64_t svxg_server_submit_device(svxg_server* S, int64_t structure, const svxg_node* nodes_dev, int32_t n,
                                  const svxg_bond* bonds_dev, int32_t nb, const svxg_material* mats_dev,
                                  const double* f_dev, const svxg_stress_options* opt, double rtol, int32_t maxit,
                                  double fragility, double* u_out, int32_t* over_out) {
  if (!S || n < 0 || nb < 0 || !mats_dev || (n > 0 && (!nodes_dev || !f_dev)) || (nb > 0 && !bonds_dev)) {
    set_error("svxg_server_submit_device: bad arguments");
    return SVXG_ERR_ARG;
  }
  Request q;
  q.structure = structure;
  q.n = n;
  q.nodes_dev = nodes_dev;
  q.bonds_dev = bonds_dev;
  q.nb_dev = nb;
  q.mats_dev = mats_dev;
  q.f_dev = f_dev;
  q.opt = opt ? *opt : svxg_default_options();
  q.rtol = rtol;
  q.maxit = maxit;
  q.fragility = fragility;
  q.u_out = u_out;
  q.over_out = over_out;
  return submit(S, std::move(q));
}

int64_t svxg_server_submit_repeat_device(svxg_server* S, int64_t structure, const int32_t* remove, int32_t nremove,
                                         const double* f_dev, int32_t n, double rtol, int32_t maxit,
                                         double fragility, double* u_out, int32_t* over_out) {
  if (!S || structure < 0 || nremove < 0 || (nremove > 0 && !remove) || n < 0 || (n > 0 && !f_dev)) {
    set_error("svxg_server_submit_repeat_device: bad arguments");
    return SVXG_ERR_ARG;
  }
  Request q;
  q.structure = structure;
  q.repeat = true;
  q.n = n;
  q.remove.assign(remove, remove + nremove);
  q.f_dev = f_dev;
  q.rtol = rtol;
  q.maxit = maxit;
  q.fragility = fragility;
  q.u_out = u_out;
  q.over_out = over_out;
  return submit(S, std::move(q));
}

int svxg_server_set_batching(svxg_server* S, int32_t max_graphs, int32_t max_graph_nodes, int64_t max_nodes) {
  if (!S || max_graphs < 1 || max_graph_nodes < 0 || max_nodes < 0) {
    set_error("svxg_server_set_batching: bad arguments");
    return SVXG_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  S->batch_graphs = max_graphs;
  S->batch_graph_nodes = max_graph_nodes;
  S->batch_nodes = max_nodes;
  return SVXG_OK;
}

int svxg_server_hold(svxg_server* S, int32_t hold) {
  if (!S) return SVXG_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->hold = hold != 0;
  }
  S->cv_work.notify_all();
  return SVXG_OK;
}

int svxg_server_wait(svxg_server* S, int64_t ticket, svxg_request_result* out) {
  if (!S || ticket <= 0) return SVXG_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  if (ticket >= S->next_ticket) {
    set_error("svxg_server_wait: no such ticket");
    return SVXG_ERR_ARG;
  }
  S->cv_done.wait(lk, [&] { return S->done.count(ticket) > 0; });
  if (out) *out = S->done[ticket];
  S->done.erase(ticket);
  return SVXG_OK;
}

int svxg_server_drain(svxg_server* S) {
  if (!S) return SVXG_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  S->cv_done.wait(lk, [&] { return S->outstanding == 0; });
  return SVXG_OK;
}

int svxg_server_stats(svxg_server* S, svxg_serving_stats* st) {
  if (!S || !st) return SVXG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(st, 0, sizeof(*st));
  st->completed = S->completed;
  st->failed = S->failed;
  st->evictions = S->evictions;
  st->admission_waits = S->admission_waits;
  st->resident = int64_t(S->resident.size());
  st->resident_bytes = S->resident_bytes;
  st->peak_bytes = S->peak;
  st->batches = S->batches;
  st->batched_requests = S->batched_requests;
  std::vector<double> l = S->latencies;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l[std::min(l.size() - 1, size_t(q * double(l.size() - 1) + 0.5))]; };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = l.back();
  }
  if (S->any) st->wall_s = std::chrono::duration<double>(S->t_last - S->t_first).count();
  return SVXG_OK;
}

int svxg_server_reset_stats(svxg_server* S) {
  if (!S) return SVXG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  S->latencies.clear();
  S->completed = S->failed = S->evictions = S->admission_waits = 0;
  S->batches = S->batched_requests = 0;
  S->peak = S->resident_bytes + S->running_bytes;
  S->any = false;
  return SVXG_OK;
}

int64_t svxg_server_estimate_bytes(int32_t n, int32_t nb) {
  return n < 0 || nb < 0 ? SVXG_ERR_ARG : estimate_bytes(n, nb);
}

int svxg_server_forget(svxg_server* S, int64_t structure) {
  if (!S) return SVXG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->resident.find(structure);
  if (it == S->resident.end()) return SVXG_OK;
  if (S->running_structures.count(structure)) {
    it->second.forget = true;
    return SVXG_OK;
  }
  drop_resident_locked(S, it, S->admin);
  S->cv_mem.notify_all();
  return SVXG_OK;
}

int svxg_batch_solve(svxg_server* S, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                     const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats,
                     const double* const* f, const svxg_stress_options* opt, double rtol, int32_t maxit,
                     double fragility, double* const* u_out, int32_t* const* over_out,
                     svxg_request_result* results) {
  if (!S || count < 0 || (count > 0 && (!nodes || !n || !bonds || !nb || !f))) {
    set_error("svxg_batch_solve: bad arguments");
    return SVXG_ERR_ARG;
  }
  std::vector<int64_t> t(size_t(count), 0);
  int err = SVXG_OK;
  svxg_server_hold(S, 1);  // (the graphs queue together, so that slots take them in batches)
  for (int32_t i = 0; i < count; ++i) {
    t[size_t(i)] = svxg_server_submit(S, -1, nodes[i], n[i], bonds[i], nb[i], mats, f[i], opt, rtol, maxit, fragility,
                                      u_out ? u_out[i] : nullptr, over_out ? over_out[i] : nullptr);
    if (t[size_t(i)] < 0) {
      err = int(t[size_t(i)]);
      break;
    }
  }
  svxg_server_hold(S, 0);
  for (int32_t i = 0; i < count; ++i) {
    if (t[size_t(i)] <= 0) break;
    svxg_request_result r{};
    const int e = svxg_server_wait(S, t[size_t(i)], &r);
    if (e && !err) err = e;
    if (results) results[i] = r;
  }
  return err;
}


int svxg_batch_piece_rounds(svxg_server* S, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                            const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats,
                            const double* gf, double* const* f, double* const* u, const svxg_stress_options* opt,
                            const svxg_piece_options* po, int32_t* const* broken_out, uint8_t* const* modes_out,
                            int32_t* const* chips_out, svxg_piece_result* piece_results,
                            svxg_request_result* results) {
  if (!S || count < 0 || (count > 0 && (!nodes || !n || !bonds || !nb || !f || !mats))) {
    set_error("svxg_batch_piece_rounds: bad arguments");
    return SVXG_ERR_ARG;
  }
  std::vector<int64_t> t(size_t(count), 0);
  int err = SVXG_OK;
  for (int32_t i = 0; i < count; ++i)
    if (n[i] < 0 || nb[i] < 0 || (n[i] > 0 && (!nodes[i] || !f[i])) || (nb[i] > 0 && !bonds[i])) {
      set_error("svxg_batch_piece_rounds: bad piece");
      return SVXG_ERR_ARG;
    }
  // the largest pieces first (by bonds), so that the longest rounds start early and the small
  // pieces fill the slots around them; each piece's result is its own whatever the order
  std::vector<int32_t> order(static_cast<size_t>(count));
  for (int32_t i = 0; i < count; ++i) order[size_t(i)] = i;
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return nb[a] > nb[b]; });
  for (const int32_t i : order) {
    Request q;
    q.n = n[i];
    q.nodes.assign(nodes[i], nodes[i] + n[i]);
    q.bonds.assign(bonds[i], bonds[i] + nb[i]);
    q.mats.assign(mats, mats + SVXG_MAX_MATERIALS);
    q.f.assign(f[i], f[i] + 6 * size_t(n[i]));
    if (u && u[i]) q.u0.assign(u[i], u[i] + 6 * size_t(n[i]));
    q.opt = opt ? *opt : svxg_default_options();
    q.po = po ? *po : svxg_default_piece_options();
    q.gf.assign(SVXG_MAX_MATERIALS, 2000.0);
    if (gf) q.gf.assign(gf, gf + SVXG_MAX_MATERIALS);
    q.piece = true;
    q.u_out = u ? u[i] : nullptr;
    q.f_out = f[i];
    q.broken_out = broken_out ? broken_out[i] : nullptr;
    q.modes_out = modes_out ? modes_out[i] : nullptr;
    q.chips_out = chips_out ? chips_out[i] : nullptr;
    q.piece_out = piece_results ? &piece_results[i] : nullptr;
    t[size_t(i)] = submit(S, std::move(q));
    if (t[size_t(i)] < 0) {
      err = int(t[size_t(i)]);
      break;
    }
  }
  for (int32_t i = 0; i < count; ++i) {
    if (t[size_t(i)] <= 0) continue;  // (not submitted: a submission failed)
    svxg_request_result r{};
    const int e = svxg_server_wait(S, t[size_t(i)], &r);
    if (e && !err) err = e;
    if (results) results[i] = r;
  }
  return err;
}

}  // extern "C"
