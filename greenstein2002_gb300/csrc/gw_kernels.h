// Device-state layout and kernel launchers shared by the CUDA sources.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gw {

// Block size of the one-thread-per-FRU kernels (fru_stage_kernel, the
// average and seeding kernels): one warp per block, so a 12,500-FRU cell's
// 391 warps spread over all 152 SMs instead of filling a few.
constexpr int kStageThreads = 32;
// Cleft-parallel stage kernels: 8 FRUs per warp, 1 .. kMaxStageWarps warps
// per block (a launch-shape choice only: the results are the same bits).
constexpr int kMaxStageWarps = 8;
// The stage kernels use no shared memory: the FRUs' MT19937 rows are read
// and regenerated in place in global memory, so the SM's unified on-chip
// memory goes to L1, which holds the rows being drawn from.
template <typename K>
cudaError_t stage_cache_attributes(K kernel) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
}
inline int stage_blocks(int nfru, int warps) { return ((nfru + 7) / 8 + warps - 1) / warps; }
// out[] slot of the device error flag (substep limit hit)
constexpr int kOutError = 31;

enum : int {
  kFlagAdvance = 1,  // run the substep loop over [t0, tf]
  kFlagSave = 2,     // snapshot FRU state before advancing (send_save_state)
  kFlagResume = 4,   // restore the snapshot before advancing (send_resume_state)
  kFlagAvg = 8,      // also reduce the 11 output-average sums (calc_fru_avg_local)
  kFlagQueueReset = 16,  // reset the FRU queue of the packed kernel for its next launch
};
enum : int { kSeedBase = 0, kSeedReference = 1 };

// Device arrays of one cell.  SoA with row stride `stride` (>= nfru):
//   frus[5][stride]   CaJSR, CaSS1..4 (mM)
//   chan[4][stride]   packed channel states of each cleft (gw_fru_model.cuh)
//   mti[stride], mt[nfru][640] (FRU-major MT19937 rows)
//   *_s               snapshot taken at the last save
//   mt_hold/hold_epoch  copy-on-twist protection of the saved MT words
//   partials[max(nblocks, ceil(nfru/8))][16], ticket: scratch of the
//                     deterministic grid reduction
//   out[32]           [0..4] flux sums, [5..8] Jxfer,Jtr,ICa,Ito2, [16..26] averages,
//                     [31] error flag
struct DevState {
  int nfru, stride, nblocks;
  double* frus;
  uint32_t* chan;
  int* mti;
  uint32_t* mt;
  double* frus_s;
  uint32_t* chan_s;
  int* mti_s;
  uint32_t* mt_hold;
  uint32_t* hold_epoch;
  double* partials;
  unsigned* ticket;
  double* out;
  unsigned long long* substeps;
  // stage trace (null unless enabled): substeps of every FRU in the last
  // 4-lane launch, and each 8-FRU warp's begin/end global time (ns)
  uint32_t* trace_sub;
  unsigned long long* trace_ns;
  // FRU queue of the packed stage kernel: qctl[0] queue head, [1..2] counts
  // of the heavy-FRU lists by launch parity, [3] substeps of the launch,
  // [4] heavy threshold; heavy_list[2][stride]; heavy_tag[2][stride] = the
  // packed launch + 1 in which the FRU was last heavy (by launch parity)
  unsigned* qctl;
  int* heavy_list;
  uint32_t* heavy_tag;
};

struct StageParams {
  double t0, tf;
  double dep0[3], span[3], depf[3];
  double nfru_scale;
  double pca_scale;  // LCC permeability scale of the cell (1 = reference PCa)
  uint32_t epoch;
  int flags;
  uint32_t launch;  // packed launches of the cell so far
};

// Many cells in one launch (cleft-parallel kernels): cell i owns blocks
// block0[i] .. block0[i+1]-1 (8 FRUs per warp); params[i].flags < 0 means
// the cell has no operation this round; its totals go to outs[i*32 ..] in the
// layout of DevState::out.
constexpr int kBatchOutStride = 32;
struct BatchArgs {
  const DevState* cells;
  const StageParams* params;
  const int* block0;  // ncells + 1 prefix sums
  double* outs;       // [ncells][kBatchOutStride]
  int ncells;
};

cudaError_t launch_stage(const DevState& s, const StageParams& p, cudaStream_t st);
cudaError_t launch_stage4_batch(const BatchArgs& a, int nblocks, int warps, cudaStream_t st);
cudaError_t launch_stage_mixed_batch(const BatchArgs& a, int nblocks, int warps, cudaStream_t st);
// cleft-parallel variants: 4 lanes per FRU, 8 FRUs per warp, `warps` warps
// per block; FP64 (the plain method) and mixed precision (FP32 rates and
// local ODE)
cudaError_t launch_stage4(const DevState& s, const StageParams& p, int warps, cudaStream_t st);
cudaError_t launch_stage_mixed(const DevState& s, const StageParams& p, int warps, cudaStream_t st);
// packed variants: `warps` single-warp blocks whose 4-lane groups take the
// cell's FRUs from a queue (heaviest of the previous launch first); they
// advance and store the FRUs only -- the sums come from a following
// non-advancing launch with kFlagQueueReset
cudaError_t launch_stage4_packed(const DevState& s, const StageParams& p, int warps, cudaStream_t st);
cudaError_t launch_stage_mixed_packed(const DevState& s, const StageParams& p, int warps, cudaStream_t st);
cudaError_t launch_avg(const DevState& s, cudaStream_t st);
// reference-order (sequential) flux and output sums of the stored FRU states,
// one thread; the flux launch overwrites out[0..8], the average one out[16..26]
cudaError_t launch_flux_seq(const DevState& s, const StageParams& p, cudaStream_t st);
cudaError_t launch_avg_seq(const DevState& s, cudaStream_t st);
// FP64 FMA throughput of the device (TFLOP/s, best of a few launches).
cudaError_t probe_fp64(int sms, double* tflops);
// Microseconds per evaluation of the 37-state global right-hand side on one
// GPU thread and on the host.
cudaError_t probe_fcn(double* device_us, double* host_us);
// exp of n arguments on the device and with the host libm.
cudaError_t probe_exp(const double* x, double* device_y, double* host_y, int n);
// FP64 issue-cost chains on one SM (gw_diag.h, gw_probe_fp64_issue).
cudaError_t probe_fp64_issue(double* cycles);
// gw_div_rn against the hardware division on n device-drawn operand pairs.
cudaError_t probe_div(unsigned long long seed, long long n, unsigned long long* mismatches);
// fcn on one thread against fcn on a warp, for n states; and the warp's cost
cudaError_t probe_fcn_compare(const double* states, int n, double time, int clamp, double* Fs, double* Fw,
                              double* Cs, double* Cw);
cudaError_t probe_fcn_warp(double* us);
cudaError_t launch_seed(const DevState& s, int scheme, uint32_t base, cudaStream_t st);

}  // namespace gw
