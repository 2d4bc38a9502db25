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

struct Resident {
  svxg_problem* p = nullptr;
  int64_t bytes = 0;
  bool forget = false;
  std::list<int64_t>::iterator lru;
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
};

namespace {

void evict_locked(svxg_server* S, int64_t need, const Slot& slot) {
  for (auto it = S->lru.begin(); it != S->lru.end() && S->resident_bytes + S->running_bytes + need > S->budget;) {
    auto r = S->resident.find(*it);
    if (r == S->resident.end() || S->running_structures.count(*it)) {
      ++it;
      continue;
    }
    slot.lend(r->second.p);
    svxg_release(r->second.p);
    S->spare.push_back(r->second.p);
    S->resident_bytes -= r->second.bytes;
    S->resident.erase(r);
    it = S->lru.erase(it);
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
  int e = svxg_set_graph(p, q.nodes.data(), q.n, q.bonds.data(), int32_t(q.bonds.size()), q.mats.data());
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
  e = solve_nodes_host(p->P, q.f.data(), uo, q.rtol, q.maxit, kCold, &r);
  if (e) return e;
  res->iters = r.iters;
  res->converged = r.converged;
  res->breakdown = r.breakdown;
  res->rel_res = r.rel_res;
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
  const int e = solve_nodes_host(p->P, q.f.data(), q.u_out, q.rtol, q.maxit, kWarmResident, &r);
  if (e) return e;
  res->warm = 1;
  res->iters = r.iters;
  res->converged = r.converged;
  res->breakdown = r.breakdown;
  res->rel_res = r.rel_res;
  return judge_into(p, q, res);
}

// A request for structure s waits while another request for s runs: it parks in deferred[s]
// and goes back to the head of the queue when that request finishes. (A repeat submitted after
// its structure's first request therefore always finds it resident, unless it was evicted.)
void release_to_spare_locked(svxg_server* S, std::unordered_map<int64_t, Resident>::iterator it, const Slot& slot) {
  slot.lend(it->second.p);
  svxg_release(it->second.p);
  S->spare.push_back(it->second.p);
  S->resident_bytes -= it->second.bytes;
  S->lru.erase(it->second.lru);
  S->resident.erase(it);
}

void worker(svxg_server* S) {
  cudaSetDevice(S->device);
  Slot slot;
  const int slot_ok = slot.init();
  svxg_problem* own = nullptr;
  for (;;) {
    Request q;
    svxg_problem* p = nullptr;
    int64_t est = 0;
    bool keep = false, admitted = false;
    int e = SVXG_OK;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
        if (S->queue.empty()) break;
        q = std::move(S->queue.front());
        S->queue.pop_front();
        if (q.structure >= 0 && S->running_structures.count(q.structure)) {
          S->deferred[q.structure].push_back(std::move(q));
          continue;
        }
        break;
      }
      if (q.ticket == 0) break;  // (stopped, nothing left)
      if (q.structure >= 0) S->running_structures.insert(q.structure);
      if (q.repeat) {
        auto it = S->resident.find(q.structure);
        if (it == S->resident.end()) {
          set_error("repeat request: the structure is not resident");
          e = SVXG_ERR_STATE;
        } else {
          p = it->second.p;
          S->lru.erase(it->second.lru);
          it->second.lru = S->lru.insert(S->lru.end(), q.structure);
        }
      } else {
        est = estimate_bytes(q.n, int64_t(q.bonds.size()));
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
          if (keep) {
            auto old = S->resident.find(q.structure);  // (resubmitted: the new graph replaces it)
            if (old != S->resident.end()) release_to_spare_locked(S, old, slot);
            if (!S->spare.empty()) {
              p = S->spare.back();
              S->spare.pop_back();
            }
          }
        }
      }
    }
    svxg_request_result res{};
    res.queue_ms = std::chrono::duration<double, std::milli>(Clock::now() - q.submitted).count();
    if (!e && slot_ok) e = slot_ok;
    if (!e && !p && !keep) {
      if (!own) e = create_bare(&own, S->device);
      p = own;
    } else if (!e && !p) {
      e = create_bare(&p, S->device);
    }
    if (!e) {
      slot.lend(p);
      e = q.repeat ? run_repeat(p, q, &res) : run_new(p, q, &res);
    }
    res.status = e;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      if (admitted) S->running_bytes -= est;
      if (q.repeat) {
        auto it = S->resident.find(q.structure);
        if (it != S->resident.end()) {
          const int64_t b = it->second.p->P.mem.bytes;
          S->resident_bytes += b - it->second.bytes;
          it->second.bytes = b;
          if (it->second.forget || e) release_to_spare_locked(S, it, slot);  // (a failed repeat: dropped)
        }
      } else if (keep && p) {
        if (!e) {
          Resident r;
          r.p = p;
          r.bytes = p->P.mem.bytes;
          r.lru = S->lru.insert(S->lru.end(), q.structure);
          S->resident[q.structure] = r;
          S->resident_bytes += r.bytes;
        } else {
          svxg_release(p);
          S->spare.push_back(p);
        }
      } else if (p && p == own) {
        svxg_release(own);
      }
      S->peak = std::max(S->peak, S->resident_bytes + S->running_bytes);
      if (q.structure >= 0) {
        S->running_structures.erase(q.structure);
        auto d = S->deferred.find(q.structure);
        if (d != S->deferred.end()) {
          for (auto it = d->second.rbegin(); it != d->second.rend(); ++it) S->queue.push_front(std::move(*it));
          S->deferred.erase(d);
          S->cv_work.notify_all();
        }
      }
      S->cv_mem.notify_all();
    }
    record(S, q, res);
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
  for (auto& kv : S->resident) {
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
  release_to_spare_locked(S, it, S->admin);
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
  for (int32_t i = 0; i < count; ++i) {
    t[size_t(i)] = svxg_server_submit(S, -1, nodes[i], n[i], bonds[i], nb[i], mats, f[i], opt, rtol, maxit, fragility,
                                      u_out ? u_out[i] : nullptr, over_out ? over_out[i] : nullptr);
    if (t[size_t(i)] < 0) {
      err = int(t[size_t(i)]);
      break;
    }
  }
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
  for (int32_t i = 0; i < count; ++i) {
    if (n[i] < 0 || nb[i] < 0 || (n[i] > 0 && (!nodes[i] || !f[i])) || (nb[i] > 0 && !bonds[i])) {
      err = SVXG_ERR_ARG;
      set_error("svxg_batch_piece_rounds: bad piece");
      break;
    }
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
    if (t[size_t(i)] <= 0) break;
    svxg_request_result r{};
    const int e = svxg_server_wait(S, t[size_t(i)], &r);
    if (e && !err) err = e;
    if (results) results[i] = r;
  }
  return err;
}

}  // extern "C"
