// Device-resident global step: the Dormand-Prince 5(4) integrator of the 37
// global states runs on the GPU beside the FRU stages, so no host round trip
// sits inside a step, and many cells advance together in one CUDA graph.
//
// Each cell has a DpCell in device memory holding the integrator's state
// (rk_pd54m.c:29-345: y, k1..k5, the trial state, start/step/ostep, the
// accept/reject state) and the parameters of its next FRU launch.  One
// "round" is two kernels: dp_round_kernel runs, for every cell at once, the
// FRU work its integrator asked for (a flux-only evaluation at an attempt's
// start, or one of stages 2..6, with the output averages fused in when an
// output step has just ended), then dp_step_kernel (one thread per cell)
// evaluates the global right-hand side (fcn.c, gw_cell_model.h) on the
// cell's flux totals and advances its integrator to the next launch.  The
// integrator stays out of the FRU kernel so as not to raise its register
// count.  A graph WHILE node repeats rounds until every cell has run its
// output steps: the whole run is one graph launch.
//
// The arithmetic is the host integrator's (gw_dp.c), operation for operation
// (compiled with -fmad=false); the results differ from the host path only
// where CUDA's exp/pow/log/fmod and the host C library round differently in
// the last place.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <new>
#include <vector>

#include "gw_cell_model.h"
#include "gw_ctx_impl.h"
#include "gw_dp_device.cuh"
#include "gw_fru.h"
#include "gw_fru_cleft.cuh"

extern "C" int gw_internal_error(int code, const char* msg);

namespace gw {

struct DpArgs {
  const DevState* cells;
  DpCell* dp;
  const int* block0;
  int ncells;
  unsigned* round_done;  // blocks of dp_step_kernel finished with this round
  unsigned* running;     // cells with output steps left
  unsigned long long* rounds;
  unsigned long long max_rounds;  // bound on the WHILE loop (a cell that never finishes is an error)
  cudaGraphConditionalHandle handle;
};

// FRU work of one round: every cell's requested launch, totals to its out[]
// slots ([0..4] flux numerators, [5..8] currents, [16..26] averages).
struct RoundFin {
  double* out;
  __device__ void operator()(const double tot[5], const double cur[4], const double* avg) const {
#pragma unroll
    for (int k = 0; k < 5; k++) out[k] = tot[k];
#pragma unroll
    for (int k = 0; k < 4; k++) out[5 + k] = cur[k];
    if (avg)
#pragma unroll
      for (int k = 0; k < 11; k++) out[16 + k] = avg[k];
  }
  __device__ void error() const { out[kOutError] = 1.0; }
};

template <typename R>
__global__ void __launch_bounds__(kMaxStageWarps * 32) dp_round_kernel(DpArgs a) {
  int lo = 0, hi = a.ncells - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&a.block0[mid]) <= b) lo = mid;
    else hi = mid - 1;
  }
  const DpCell* c = a.dp + lo;
  if (c->done || c->err) return;  // uniform over the block (one cell per block)
  const DevState& s = a.cells[lo];
  const StageParams& p = c->sp;
  cleft::stage_body_fin<R>(s, p, b - a.block0[lo], RoundFin{s.out});
}

// The integrators of all cells, one thread each; the last block to finish
// decides whether another round runs.
__global__ void __launch_bounds__(32) dp_step_kernel(DpArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.ncells) {
    DpCell& c = a.dp[i];
    if (!c.done && !c.err) {
      double* o = a.cells[i].out;
      if (o[kOutError] != 0.0) {
        c.err = 1;  // substep limit: corrupted FRU state
        atomicSub(a.running, 1u);
      } else {
        const double* avg = (c.sp.flags & kFlagAvg) ? o + 16 : nullptr;
        const double J[4] = {o[5], o[6], o[7], o[8]};
        dp_after(c, J, avg);
        if (c.done || c.err) atomicSub(a.running, 1u);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.round_done, 1u) == gridDim.x - 1u) {
      __threadfence();
      *a.round_done = 0u;
      const unsigned long long r = *a.rounds + 1ull;
      *a.rounds = r;
      const bool more = *(volatile unsigned*)a.running > 0u && r < a.max_rounds;
      cudaGraphSetConditional(a.handle, more ? 1u : 0u);
    }
  }
}

}  // namespace gw

using gw::DpCell;

extern "C" int gw_run_device(int n, gw_ctx** cells, const gw_settings* sets, double* t, double* states,
                             double* oldsteps, int n_steps, double* state_trace, double* other_trace,
                             double* cur_trace) {
  if (n <= 0 || !cells || !sets || !t || !states || !oldsteps || n_steps <= 0)
    return gw_internal_error(GW_EINVAL, "gw_run_device: bad argument");
  const int prec = cells[0]->precision;
  for (int i = 0; i < n; i++)
    if (!cells[i] || cells[i]->precision != prec || cells[i]->fru_lanes != 4 || cells[i]->batch ||
        cells[i]->sum_order != GW_SUM_TREE)
      return gw_internal_error(GW_EINVAL,
                               "gw_run_device: cells must share one precision, use the 4-lane kernel and tree-order "
                               "sums and not be batched");
  const int warps = cells[0]->stage_warps;
  std::vector<gw::DevState> hcells(n);
  std::vector<int> hblock0(n + 1);
  std::vector<DpCell> hdp(n);
  int acc = 0;
  for (int i = 0; i < n; i++) {
    gw_ctx* c = cells[i];
    cudaStreamSynchronize(c->stream);
    hcells[i] = c->d;
    hblock0[i] = acc;
    acc += gw::stage_blocks(c->d.nfru, warps);
    DpCell& d = hdp[i];
    memset(&d, 0, sizeof d);
    memcpy(d.y, states + (size_t)i * GW_NSTATE, sizeof d.y);
    d.set = sets[i];
    d.tnow = t[i];
    d.oldstep = oldsteps[i];
    d.epoch = c->epoch;
    d.pending = c->pending;
    d.steps_left = n_steps;
    d.nfru = c->d.nfru;
    d.sp.nfru_scale = c->nfru_scale;
    d.sp.pca_scale = c->pca_scale;
  }
  hblock0[n] = acc;
  const size_t ns = (size_t)n * n_steps;
  gw::DevState* dcells = nullptr;
  int* dblock0 = nullptr;
  DpCell* ddp = nullptr;
  unsigned* dcount = nullptr;  // [0] round_done, [1] running
  unsigned long long* drounds = nullptr;
  double *dst = nullptr, *dot = nullptr, *dcu = nullptr;
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int rc = GW_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&dcells, sizeof(gw::DevState) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dblock0, sizeof(int) * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&ddp, sizeof(DpCell) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dcount, sizeof(unsigned) * 2);
  if (e == cudaSuccess) e = cudaMalloc(&drounds, sizeof(unsigned long long));
  if (e == cudaSuccess && state_trace) e = cudaMalloc(&dst, sizeof(double) * ns * GW_NSTATE);
  if (e == cudaSuccess && other_trace) e = cudaMalloc(&dot, sizeof(double) * ns * GW_NOTHER);
  if (e == cudaSuccess && cur_trace) e = cudaMalloc(&dcu, sizeof(double) * ns * GW_NCUR);
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    DpCell& d = hdp[i];
    d.tr_states = dst ? dst + (size_t)i * n_steps * GW_NSTATE : nullptr;
    d.tr_other = dot ? dot + (size_t)i * n_steps * GW_NOTHER : nullptr;
    d.tr_cur = dcu ? dcu + (size_t)i * n_steps * GW_NCUR : nullptr;
  }
  // the first launch of every cell: the flux at its first attempt's start
  // (the integrator's own arithmetic runs on the device from then on)
  if (e == cudaSuccess) {
    std::vector<DpCell> init = hdp;
    for (int i = 0; i < n; i++) {
      DpCell& d = init[i];
      d.tstep = d.tnow + d.set.time_step;
      double step = d.oldstep < d.tstep - d.tnow ? d.oldstep : d.tstep - d.tnow;
      step = d.set.step_max < step ? d.set.step_max : step;
      d.step = step;
      d.ostep = step;
      d.start = d.tnow;
      d.success = 1;
      d.keepc = 1;
      d.phase = gw::kPhFlux;
      d.sp.t0 = d.sp.tf = 0.0;
      const double dep[3] = {d.y[GW_V], d.y[GW_Cai], d.y[GW_CaNSR]};
      for (int k = 0; k < 3; k++) {
        d.sp.dep0[k] = d.sp.depf[k] = dep[k];
        d.sp.span[k] = 0.0;
      }
      d.sp.epoch = d.epoch;
      d.sp.flags = d.pending;
      d.pending = 0;
    }
    const unsigned cnt[2] = {0u, (unsigned)n};
    e = cudaMemcpyAsync(ddp, init.data(), sizeof(DpCell) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dcells, hcells.data(), sizeof(gw::DevState) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dblock0, hblock0.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dcount, cnt, sizeof cnt, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(drounds, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  // graph: WHILE (cells running) { one round }
  gw::DpArgs args;
  args.cells = dcells;
  args.dp = ddp;
  args.block0 = dblock0;
  args.ncells = n;
  args.round_done = dcount;
  args.running = dcount + 1;
  args.rounds = drounds;
  // far above any real run (tens to hundreds of rounds per simulated ms)
  args.max_rounds = 100000ull * (unsigned long long)n_steps + 1000ull;
  if (e == cudaSuccess) e = cudaGraphCreate(&graph, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&args.handle, graph, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams cp = {};
  cudaGraphNode_t cnode, knode;
  if (e == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = args.handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&cnode, graph, nullptr, nullptr, 0, &cp);
  }
  if (e == cudaSuccess) {
    void* kfun = prec == 1 ? (void*)gw::dp_round_kernel<float> : (void*)gw::dp_round_kernel<double>;
    e = prec == 1 ? gw::stage_cache_attributes(gw::dp_round_kernel<float>)
                  : gw::stage_cache_attributes(gw::dp_round_kernel<double>);
    void* kargs[] = {&args};
    cudaGraphNodeParams kp = {};
    kp.type = cudaGraphNodeTypeKernel;
    kp.kernel.func = kfun;
    kp.kernel.gridDim = dim3(acc);
    kp.kernel.blockDim = dim3(32 * warps);
    kp.kernel.sharedMemBytes = 0;
    kp.kernel.kernelParams = kargs;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (e == cudaSuccess) e = cudaGraphAddNode(&knode, body, nullptr, nullptr, 0, &kp);
    cudaGraphNodeParams sp = {};
    sp.type = cudaGraphNodeTypeKernel;
    sp.kernel.func = (void*)gw::dp_step_kernel;
    sp.kernel.gridDim = dim3((n + 31) / 32);
    sp.kernel.blockDim = dim3(32);
    sp.kernel.sharedMemBytes = 0;
    sp.kernel.kernelParams = kargs;
    cudaGraphNode_t snode;
    if (e == cudaSuccess) e = cudaGraphAddNode(&snode, body, &knode, nullptr, 1, &sp);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  unsigned long long rounds = 0;
  if (e == cudaSuccess) e = cudaMemcpy(hdp.data(), ddp, sizeof(DpCell) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&rounds, drounds, sizeof rounds, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dst) e = cudaMemcpy(state_trace, dst, sizeof(double) * ns * GW_NSTATE, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dot) e = cudaMemcpy(other_trace, dot, sizeof(double) * ns * GW_NOTHER, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dcu) e = cudaMemcpy(cur_trace, dcu, sizeof(double) * ns * GW_NCUR, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    rc = gw_internal_error(GW_ECUDA, cudaGetErrorString(e));
  } else {
    for (int i = 0; i < n; i++) {
      const DpCell& d = hdp[i];
      if (d.err || !d.done) {
        rc = gw_internal_error(GW_EINVAL, d.err == 1   ? "gw_run_device: substep limit reached (corrupted FRU state)"
                                          : d.err == 2 ? "gw_run_device: global state not finite"
                                                       : "gw_run_device: a cell did not finish its output steps");
        break;
      }
      memcpy(states + (size_t)i * GW_NSTATE, d.y, sizeof d.y);
      t[i] = d.tnow;
      oldsteps[i] = d.oldstep;
      cells[i]->epoch = d.epoch;
      cells[i]->pending = 0;
      cells[i]->launches += 2 * rounds;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaFree(dcells);
  cudaFree(dblock0);
  cudaFree(ddp);
  cudaFree(dcount);
  cudaFree(drounds);
  cudaFree(dst);
  cudaFree(dot);
  cudaFree(dcu);
  if (st) cudaStreamDestroy(st);
  return rc;
}
