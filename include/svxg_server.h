/* svxg_server.h - many stress solves in flight on one GPU: the serving loop and the batched solve.
 *
 * The reference solves many independent graphs at once only on the host: piece checks call
 * distinct StressProblem objects from pool threads, one graph per thread under SerialScope
 * (core/src/world/world_pieces.cpp:1460-1463). This is that pattern for a GPU-resident solve,
 * plus what a request loop needs: admission against an HBM budget, structures kept resident
 * between requests (K, the multigrid hierarchy and the last displacement stay on the device),
 * warm-started repeat solves after in-place bond removal, and per-request latency.
 *
 * A server owns `workers` host threads (its slots). Each takes the oldest waiting request, runs
 * it on a problem of its own (its own CUDA stream: the solves of different requests overlap on
 * the device) and records the result under the request's ticket. A new structure is admitted
 * when the bytes of the resident structures, of the requests running and of its own estimate
 * fit in the budget; resident structures no request is using are evicted, least recently used
 * first, to make room.
 *
 * Batching: a slot that takes a new request also takes the new requests queued behind it with the
 * same options (up to a number of graphs and of nodes, svxg_server_set_batching) and runs them as
 * one problem (svxg_set_graphs: every launch covers the batch, each graph stops at its own
 * target); a batch whose structures are kept stays resident as one problem (a bundle), and a
 * repeat of one of them - with the repeats of other members queued behind it - removes its bonds
 * in place and solves the bundle warm. A request run alone gives the single-problem entry points'
 * result bit for bit; in a batch, every graph meets the same tolerance (||r_g|| <= rtol ||f_g||)
 * and gives the same result within it.
 */
#ifndef SVXG_SERVER_H
#define SVXG_SERVER_H

#include "svxg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct svxg_server svxg_server;

/* A finished request. 64 bytes. */
typedef struct svxg_request_result {
  int64_t ticket;
  int32_t status;     /* SVXG_OK, or the error of the step that failed */
  int32_t iters, converged, breakdown;
  int32_t failing;    /* bonds with phi >= 1 after the solve */
  int32_t warm;       /* 1: started from the structure's last solution on the device */
  double rel_res;
  double queue_ms;    /* submission -> a slot took it */
  double latency_ms;  /* submission -> result recorded */
  double err_est;     /* the solve's error estimate under the mixed-precision policy (svxg_info) */
} svxg_request_result;

/* Counters since creation (or the last reset). 112 bytes. */
typedef struct svxg_serving_stats {
  int64_t completed, failed, evictions, admission_waits;
  int64_t resident, resident_bytes, peak_bytes; /* structures kept, their bytes, peak admitted bytes */
  int64_t pad;
  double p50_ms, p99_ms, max_ms; /* request latency */
  double wall_s;                 /* first submission -> last completion */
  int64_t batches, batched_requests; /* batches of new requests run, the requests in them */
} svxg_serving_stats;

/* A server on `device` with `workers` slots admitting up to `hbm_budget_bytes` of problem memory. */
int svxg_server_create(svxg_server** out, int device, int64_t hbm_budget_bytes, int32_t workers);
/* Finishes the requests already submitted, then frees everything. */
void svxg_server_destroy(svxg_server* s);

/* A solve of a new graph: assemble (options `opt`, null: defaults), solve from zero to `rtol`
 * (maxit < 0: no cap), judge at `fragility`. The graph, material table and load are copied;
 * u_out (6 n doubles) and over_out (nb int32: the failing bonds, ascending) may be null, and
 * must stay valid until the request is waited for. structure >= 0 keeps the problem resident
 * under that id (replacing an earlier one) for repeat requests. Returns a ticket (> 0) or an
 * error code (< 0). */
int64_t svxg_server_submit(svxg_server* s, int64_t structure, const svxg_node* nodes, int32_t n,
                           const svxg_bond* bonds, int32_t nb, const svxg_material* mats, const double* f,
                           const svxg_stress_options* opt, double rtol, int32_t maxit, double fragility,
                           double* u_out, int32_t* over_out);

/* A repeat solve of resident structure `structure`: remove the listed bonds in place (the
 * reference's remove_bond: K downdated, the preconditioner kept), solve from the structure's last
 * solution, judge. n: its node count (f: 6 n doubles). A structure evicted or never kept returns
 * status SVXG_ERR_STATE in its result: submit the graph again. */
int64_t svxg_server_submit_repeat(svxg_server* s, int64_t structure, const int32_t* remove, int32_t nremove,
                                  const double* f, int32_t n, double rtol, int32_t maxit, double fragility,
                                  double* u_out, int32_t* over_out);

/* The same two submissions with the graph, the material table and the load in device memory of the
 * server's device (svxg_set_graph_device), read when the request runs: they must stay valid and
 * unchanged until the request is waited for. u_out may be device or host memory; over_out is host
 * memory. */
int64_t svxg_server_submit_device(svxg_server* s, int64_t structure, const svxg_node* nodes_dev, int32_t n,
                                  const svxg_bond* bonds_dev, int32_t nb, const svxg_material* mats_dev,
                                  const double* f_dev, const svxg_stress_options* opt, double rtol, int32_t maxit,
                                  double fragility, double* u_out, int32_t* over_out);
int64_t svxg_server_submit_repeat_device(svxg_server* s, int64_t structure, const int32_t* remove, int32_t nremove,
                                         const double* f_dev, int32_t n, double rtol, int32_t maxit,
                                         double fragility, double* u_out, int32_t* over_out);

/* Batching of new requests: at most max_graphs graphs (1: none), each of at most max_graph_nodes
 * nodes, max_nodes in all, per problem. Defaults 16, 20,000 and 65,536. */
int svxg_server_set_batching(svxg_server* s, int32_t max_graphs, int32_t max_graph_nodes, int64_t max_nodes);
/* hold != 0: slots finish what they run and take no new request (submissions queue); 0: they take
 * the queue again - a caller that submits a frame's requests together and releases them gets them
 * batched. Destroying the server runs what is queued, held or not. */
int svxg_server_hold(svxg_server* s, int32_t hold);

/* Blocks until the ticket's request has finished; its result is handed over once. */
int svxg_server_wait(svxg_server* s, int64_t ticket, svxg_request_result* out);
/* Blocks until every submitted request has finished. */
int svxg_server_drain(svxg_server* s);
int svxg_server_stats(svxg_server* s, svxg_serving_stats* out);
int svxg_server_reset_stats(svxg_server* s);
/* The bytes admission reserves for a new structure of n nodes and nb bonds while it runs (its
 * actual bytes replace the estimate once it is resident). */
int64_t svxg_server_estimate_bytes(int32_t n, int32_t nb);
/* Drops a resident structure (no effect while a request uses it: it is dropped afterwards). */
int svxg_server_forget(svxg_server* s, int64_t structure);

/* The batched solve: `count` independent graphs (arrays of per-graph pointers and sizes; one
 * material table), each assembled, solved from zero and judged as a request of `s`, all queued
 * together (the slots held while they are submitted, then released: any earlier hold ends), so
 * that the slots take them in batches; returns when all have finished. u_out and over_out (arrays
 * of per-graph buffers) may be null. */
int svxg_batch_solve(svxg_server* s, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                     const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats,
                     const double* const* f, const svxg_stress_options* opt, double rtol, int32_t maxit,
                     double fragility, double* const* u_out, int32_t* const* over_out,
                     svxg_request_result* results);

/* A substep's loose pieces (World::Impl::body_stress_run for each, core/src/world/world_pieces.cpp
 * :614-808, which the reference runs one piece per pool thread): `count` pieces, each its own
 * graph with its load f[i] (6 n[i], in and out: the chips' loads move), warm start and result in
 * u[i] (may be null: from rest, not returned), run through svxg_piece_rounds as requests of `s`
 * (all in flight at once over its slots). broken_out / modes_out (nb[i] entries each) and
 * chips_out (n[i]) may be null; piece_results and results (count entries) may be null. */
int svxg_batch_piece_rounds(svxg_server* s, int32_t count, const svxg_node* const* nodes, const int32_t* n,
                            const svxg_bond* const* bonds, const int32_t* nb, const svxg_material* mats,
                            const double* gf, double* const* f, double* const* u, const svxg_stress_options* opt,
                            const svxg_piece_options* po, int32_t* const* broken_out, uint8_t* const* modes_out,
                            int32_t* const* chips_out, svxg_piece_result* piece_results,
                            svxg_request_result* results);

#ifdef __cplusplus
}
#endif

#endif /* SVXG_SERVER_H */
