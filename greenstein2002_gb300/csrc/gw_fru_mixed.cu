// Mixed-precision cleft-parallel FRU stage kernel: transition rates and the
// FRU-local Ca ODE in FP32 (FP32 issues 64x faster than FP64 on GB300); the
// FRU Ca state, the FRU clock, its step and the cross-FRU flux sums stay FP64.
// The channel algorithm, its MT19937 draw order and the transition rules are
// the FP64 method's (gw_fru_cleft.cuh), so both share every random number.
//
// Reference: simfru_local.c:32-278, fru_rates_local.c:30-798, fcn_fru.c:23-137.
#include "gw_fru_cleft.cuh"

namespace gw {

__global__ void __launch_bounds__(kMaxStageWarps * 32) fru_stage_mixed_kernel(DevState s, StageParams p) {
  cleft::stage_body<float>(s, p, blockIdx.x, s.out);
}

cudaError_t launch_stage_mixed(const DevState& s, const StageParams& p, int warps, cudaStream_t st) {
  const int blocks = stage_blocks(s.nfru, warps);
  static const cudaError_t attr = stage_cache_attributes(fru_stage_mixed_kernel);
  if (attr != cudaSuccess) return attr;
  fru_stage_mixed_kernel<<<blocks, 32 * warps, 0, st>>>(s, p);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(kMaxStageWarps * 32) fru_stage_mixed_batch_kernel(BatchArgs a) { cleft::batch_body<float>(a); }

cudaError_t launch_stage_mixed_batch(const BatchArgs& a, int nblocks, int warps, cudaStream_t st) {
  static const cudaError_t attr = stage_cache_attributes(fru_stage_mixed_batch_kernel);
  if (attr != cudaSuccess) return attr;
  fru_stage_mixed_batch_kernel<<<nblocks, 32 * warps, 0, st>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(32, 16) fru_stage_mixed_packed_kernel(DevState s, StageParams p) {
  cleft::stage_body_packed<float>(s, p, s.out);
}

cudaError_t launch_stage_mixed_packed(const DevState& s, const StageParams& p, int warps, cudaStream_t st) {
  static const cudaError_t attr = stage_cache_attributes(fru_stage_mixed_packed_kernel);
  if (attr != cudaSuccess) return attr;
  fru_stage_mixed_packed_kernel<<<warps, 32, 0, st>>>(s, p);
  return cudaGetLastError();
}

}  // namespace gw
