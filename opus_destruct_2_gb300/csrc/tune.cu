// tune.cu - the row schedule of every BSR operator, chosen from the committed table.
//
// The two schedules of spmv_row.cuh add a row's blocks in different orders, and the reductions
// fused into the conjugate-gradient products group rows by thread block differently. The choice
// is therefore a fixed function of the operator's shape (mean blocks per row against the bound of
// sched_table.h), never of a timing, so a problem gives the same bits alone, among other problems,
// and from one run to the next.
// The table is fitted offline by opus_destruct_2_gb300/autotune.py from the timings this file
// records when asked.
#include <chrono>
#include <cstdlib>

#include "problem.cuh"
#include "sched_table.h"
#include "spmv_row.cuh"

namespace svxg {

namespace {
int env_level() {
  const char* live = std::getenv("SVXG_TUNE_LIVE");
  if (live && live[0] && live[0] != '0') return 2;
  const char* log = std::getenv("SVXG_TUNE_LOG");
  return log && log[0] && log[0] != '0' ? 1 : 0;
}
const int g_level = env_level();
}  // namespace

int table_sched(int kind, int64_t rows, int64_t blocks) {
  if (rows <= 0 || kind < 0 || kind > 3) return kWarpRow;
  return double(blocks) / double(rows) <= kGroupRowMaxMean[kind] ? kGroupRow : kWarpRow;
}

bool tune_timing() { return g_level > 0; }

namespace {
const bool g_trace = [] {
  const char* v = std::getenv("SVXG_TRACE");
  return v && v[0] && v[0] != '0';
}();
double now_us() {
  return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

void trace_mark(Problem& P, const char* label, bool restart) {
  if (P.phase_on) {
    if (restart) P.phase_used = 0;
    if (P.phase_used == P.phase_events.size()) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) == cudaSuccess) {
        P.phase_events.push_back(e);
        P.phase_labels.push_back(nullptr);
      }
    }
    if (P.phase_used < P.phase_events.size() && cudaEventRecord(P.phase_events[P.phase_used], P.stream) == cudaSuccess)
      P.phase_labels[P.phase_used++] = label;
  }
  if (!g_trace) return;
  cudaStreamSynchronize(P.stream);
  const double t = now_us();
  if (restart || P.trace.empty()) {
    P.trace.clear();
    P.trace.emplace_back("start", t);
    if (restart) return;
  }
  P.trace.emplace_back(label, t);
}

int tune_decide(Problem& P, int kind, int level, int64_t rows, int64_t blocks, float ms_warp, float ms_group) {
  svxg_tune_entry e{};
  e.kind = kind;
  e.level = level;
  e.rows = rows;
  e.blocks = blocks;
  e.ms_warp_row = ms_warp;
  e.ms_group_row = ms_group;
  P.tune_log.push_back(e);
  if (g_level == 2) return ms_group < ms_warp ? kGroupRow : kWarpRow;
  return table_sched(kind, rows, blocks);
}

// FP64 throughput of this GPU: every thread runs kChains independent FMA chains (enough in flight
// to cover the pipe's latency at 8 warps a scheduler), the grid a multiple of the SM count. The
// chains' values are written only when a flag no caller sets is on, so nothing is optimized away.
namespace {
constexpr int kChains = 16;
__global__ void __launch_bounds__(256) k_dfma_rate(int32_t iters, double m, double c, int32_t write, double* out) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = 1e-3 * double(threadIdx.x + k);
  for (int32_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], m, c);
  }
  double t = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) t += a[k];
  if (write) out[blockIdx.x * blockDim.x + threadIdx.x] = t;
}
}  // namespace

int measure_fp64_rate(int device, double* tflops) {
  *tflops = 0.0;
  int sms = 0;
  SVXG_CUDA(cudaSetDevice(device));
  SVXG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const unsigned blocks = unsigned(sms) * 8u;
  const int32_t iters = 4096;
  cudaStream_t st;
  SVXG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  SVXG_CUDA(cudaEventCreate(&e0));
  SVXG_CUDA(cudaEventCreate(&e1));
  float best = 0.0f;
  for (int r = 0; r < 6; ++r) {
    SVXG_CUDA(cudaEventRecord(e0, st));
    (k_dfma_rate<<<blocks, 256, 0, st>>>(iters, 0.999999, 1e-9, 0, nullptr), SVXG_COUNT_LAUNCH());
    SVXG_CUDA(cudaEventRecord(e1, st));
    SVXG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    SVXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (r > 0 && (best == 0.0f || ms < best)) best = ms;  // (the first launch warms up)
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  SVXG_CUDA(cudaGetLastError());
  const double flops = 2.0 * kChains * double(iters) * double(blocks) * 256.0;
  *tflops = best > 0.0f ? flops / (double(best) * 1e-3) / 1e12 : 0.0;
  return SVXG_OK;
}

}  // namespace svxg

