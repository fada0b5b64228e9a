// FP64 cleft-parallel FRU stage kernel (the plain method): the substep loop
// of gw_fru_cleft.cuh instantiated in double.  Compiled with -fmad=false so
// every floating-point operation is the reference's own, rounded once.
//
// Reference: simfru_local.c:32-278 (see gw_fru_cleft.cuh for the mapping).
#include "gw_fru_cleft.cuh"

namespace gw {

__global__ void __launch_bounds__(kMaxStageWarps * 32) fru_stage4_kernel(DevState s, StageParams p) {
  cleft::stage_body<double>(s, p, blockIdx.x, s.out);
}

cudaError_t launch_stage4(const DevState& s, const StageParams& p, int warps, cudaStream_t st) {
  const int blocks = stage_blocks(s.nfru, warps);
  static const cudaError_t attr = stage_cache_attributes(fru_stage4_kernel);
  if (attr != cudaSuccess) return attr;
  fru_stage4_kernel<<<blocks, 32 * warps, 0, st>>>(s, p);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(kMaxStageWarps * 32) fru_stage4_batch_kernel(BatchArgs a) { cleft::batch_body<double>(a); }

cudaError_t launch_stage4_batch(const BatchArgs& a, int nblocks, int warps, cudaStream_t st) {
  static const cudaError_t attr = stage_cache_attributes(fru_stage4_batch_kernel);
  if (attr != cudaSuccess) return attr;
  fru_stage4_batch_kernel<<<nblocks, 32 * warps, 0, st>>>(a);
  return cudaGetLastError();
}

// At least eleven single-warp blocks per SM: the register cap (<= 186 per
// thread; 168 used, so twelve fit) against 191 uncapped (measured 4-13%
// faster on the 16-cell ensemble, where the FP64 pipe is ~75% busy).
__global__ void __launch_bounds__(32, 11) fru_stage4_packed_kernel(DevState s, StageParams p) {
  cleft::stage_body_packed<double>(s, p, s.out);
}

cudaError_t launch_stage4_packed(const DevState& s, const StageParams& p, int warps, cudaStream_t st) {
  static const cudaError_t attr = stage_cache_attributes(fru_stage4_packed_kernel);
  if (attr != cudaSuccess) return attr;
  fru_stage4_packed_kernel<<<warps, 32, 0, st>>>(s, p);
  return cudaGetLastError();
}

}  // namespace gw
