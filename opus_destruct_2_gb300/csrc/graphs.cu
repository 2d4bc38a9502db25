// graphs.cu - a whole iterate() as one CUDA graph launch.
//
// One iteration of the conjugate-gradient sequence (SpMV, updates, the full V-cycle, r.z, the p
// update) is captured once per assembled problem into the body of a WHILE conditional node; a
// last kernel in the body sets the node's condition from the run's device-side done flag. A
// launch therefore runs iterations until convergence, breakdown or the cap with no host round
// trip and no per-kernel launch cost (kernels already inside a graph), instead of the host's
// batches of launches and flag reads.
#include <cuda_runtime.h>

#include "problem.cuh"

namespace svxg {

void uncount_launches(int64_t n);

namespace {

__global__ void k_loop_cond(cudaGraphConditionalHandle h, const int32_t* done) {
  if (threadIdx.x == 0) cudaGraphSetConditional(h, *done ? 0u : 1u);
}

}  // namespace

struct LoopGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t body_launches = 0;
};

void destroy_loop(void*& slot) {
  LoopGraph* L = static_cast<LoopGraph*>(slot);
  if (!L) return;
  if (L->exec) cudaGraphExecDestroy(L->exec);
  if (L->graph) cudaGraphDestroy(L->graph);
  delete L;
  slot = nullptr;
}

// Builds (once) and launches the loop graph in `slot`: body() enqueues one iteration on P.stream;
// `done` is the device flag that ends the loop. Returns the body's launch count in *body_launches.
int run_loop(Problem& P, void*& slot, const int32_t* done, int (*body)(Problem&), int64_t* body_launches) {
  if (P.nfree <= 0) {
    set_error("loop graph: no free DOFs");
    return SVXG_ERR_STATE;
  }
  LoopGraph* L = static_cast<LoopGraph*>(slot);
  if (!L) {
    L = new LoopGraph;
    slot = L;
    SVXG_CUDA(cudaGraphCreate(&L->graph, 0));
    cudaGraphConditionalHandle h;
    SVXG_CUDA(cudaGraphConditionalHandleCreate(&h, L->graph, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    SVXG_CUDA(cudaGraphAddNode(&node, L->graph, nullptr, nullptr, 0, &np));
    cudaGraph_t body_graph = np.conditional.phGraph_out[0];
    SVXG_CUDA(cudaStreamBeginCaptureToGraph(P.stream, body_graph, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal));
    // (counted on this thread: slots on other threads launch meanwhile)
    const int64_t c0 = thread_launch_count();
    int e = body(P);
    if (!e) {
      (k_loop_cond<<<1, 32, 0, P.stream>>>(h, done), SVXG_COUNT_LAUNCH());
      if (cudaGetLastError() != cudaSuccess) e = SVXG_ERR_CUDA;
    }
    cudaGraph_t captured = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(P.stream, &captured);
    L->body_launches = thread_launch_count() - c0;
    uncount_launches(L->body_launches);  // (captured, not run)
    if (e || ce != cudaSuccess) {
      if (ce != cudaSuccess) set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
      destroy_loop(slot);
      return e ? e : SVXG_ERR_CUDA;
    }
    SVXG_CUDA(cudaGraphInstantiate(&L->exec, L->graph, 0));
  }
  SVXG_CUDA(cudaGraphLaunch(L->exec, P.stream));
  if (body_launches) *body_launches = L->body_launches;
  return SVXG_OK;
}

}  // namespace svxg
