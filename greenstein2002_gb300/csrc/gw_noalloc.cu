// Allocation-free FRU stage: advance FRU arrays that the caller owns on the
// device over one stage interval and reduce their fluxes, without allocating
// any memory.
//
// Who needs it: callers that must not call cudaMalloc while they run.
// cudaMalloc synchronises the whole device (stalling every other stream of a
// serving loop that overlaps many cells), is not allowed while a stream is
// being captured into a CUDA graph, and is off limits to plug-in hosts that
// hand out all device memory from their own fixed pool.  Such callers already
// hold the FRU arrays; what the stage kernel still needs beyond them is a
// small reduction scratch (per-block partial sums and a completion ticket).
// Here that scratch is a file-scope __device__ array of fixed size, present
// on every GPU that loads the library until the process exits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_fru.h"
#include "gw_fru_core.cuh"

namespace gw {

// Largest cell this entry point accepts, and its scratch: per-block partial
// sums (5 doubles per 32-FRU block) followed by the completion ticket.
constexpr int kNoAllocMaxFru = 65536;
constexpr int kNoAllocMaxBlocks = kNoAllocMaxFru / kStageThreads;
constexpr size_t kNoAllocPartialsBytes = sizeof(double) * 5 * kNoAllocMaxBlocks;
// out[] layout of this entry point: [0..4] flux sums, [5..8] Jxfer, Jtr,
// ICa, Ito2, [9] error flag (1: substep limit reached; 2: an FRU's mti or a
// channel state was out of range, and that FRU was left untouched)
constexpr int kNoAllocOutError = 9;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocPartialsBytes + 256];

// The caller's arrays do not pass through gw_upload's checks, so the kernel
// checks what would otherwise index out of range: mti in 0..624 (the MT row)
// and each cleft's channel word (LCC 1..12, VDI 1..2, RyR 1..8, ClCh 1..2;
// the rate tables).
__device__ __forceinline__ bool noalloc_valid(int mti, const uint32_t w[kClefts]) {
  bool ok = mti >= 0 && mti <= kMtN;
#pragma unroll
  for (int c = 0; c < kClefts; c++) {
    const int l = lcc_of(w[c]), v = vdi_of(w[c]), x = cl_of(w[c]);
    ok = ok && l >= 1 && l <= 12 && v >= 1 && v <= 2 && x >= 1 && x <= 2;
#pragma unroll
    for (int i = 0; i < kRyR; i++) {
      const int r = ryr_of(w[c], i);
      ok = ok && r >= 1 && r <= 8;
    }
  }
  return ok;
}

// Copy-on-twist is off here: the hold epoch word always equals the epoch the
// kernel is launched with, so a regeneration never copies words aside (no
// save/resume on this path).
constexpr uint32_t kNoHoldEpoch = 0u;

__global__ void __launch_bounds__(kStageThreads)
fru_stage_noalloc_kernel(int nfru, int stride, double* frus, uint32_t* chan, int* mti, uint32_t* mt,
                         StageParams p, double* partials, unsigned* ticket, double* out) {
  __shared__ double smem[32 * 5];
  __shared__ uint32_t no_hold_epoch;
  if (threadIdx.x == 0) no_hold_epoch = kNoHoldEpoch;
  __syncthreads();
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  bool overflow = false, invalid = false;
  if (f < nfru) {
    const size_t nf = (size_t)stride;
    double y[5];
    uint32_t w[kClefts];
    uint32_t nsub = 0;
    MtRef rng;
    rng.m = mt + (size_t)f * kMtStride;
    rng.hold = nullptr;
    rng.hold_epoch = &no_hold_epoch;
    rng.epoch = kNoHoldEpoch;
#pragma unroll
    for (int i = 0; i < 5; i++) y[i] = frus[i * nf + f];
#pragma unroll
    for (int c = 0; c < kClefts; c++) w[c] = chan[c * nf + f];
    rng.mti = mti[f];
    invalid = !noalloc_valid(rng.mti, w);
    if (!invalid) {
      advance_fru(p, y, w, rng, nsub, overflow);
#pragma unroll
      for (int i = 0; i < 5; i++) frus[i * nf + f] = y[i];
#pragma unroll
      for (int c = 0; c < kClefts; c++) chan[c * nf + f] = w[c];
      mti[f] = rng.mti;
    }
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      v[0] += y[c + 1];
      if (lcc_open(w[c])) {
        v[2] += y[c + 1];
        v[3] += 1.0;
      }
      if (cl_of(w[c]) == 2) v[4] += 1.0;
    }
    v[1] = y[0];
  }
  if (invalid) out[kNoAllocOutError] = 2.0;
  else if (overflow) out[kNoAllocOutError] = 1.0;
  block_reduce<5>(v, smem);
  double tot[5];
  if (grid_finish<5>(v, partials, ticket, smem, tot)) {
    double cur[4];
    currents_from_sums(nfru, p.nfru_scale, p.depf, tot, cur);
#pragma unroll
    for (int k = 0; k < 5; k++) out[k] = tot[k];
#pragma unroll
    for (int k = 0; k < 4; k++) out[5 + k] = cur[k];
  }
}

}  // namespace gw

// Per-device address of the scratch array, resolved once per device with
// that device current (the host-side name of a __device__ array is only a
// stand-in, not a device address).
static void* g_scratch_addr[64];

extern "C" int gw_internal_error(int code, const char* msg);

extern "C" int gw_stage_noalloc(int nfru, int stride, double* frus, uint32_t* chan, int* mti, uint32_t* mt,
                                double t0, double tf, const double dep0[3], const double depf[3], double nfru_scale,
                                double* out, void* stream) {
  using namespace gw;
  if (nfru <= 0 || nfru > kNoAllocMaxFru)
    return gw_internal_error(GW_EINVAL, "gw_stage_noalloc: nfru must be in 1..65536 (fixed scratch size)");
  if (stride < nfru || !frus || !chan || !mti || !mt || !dep0 || !depf || !out)
    return gw_internal_error(GW_EINVAL, "gw_stage_noalloc: null array or stride < nfru");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return gw_internal_error(GW_ECUDA, "gw_stage_noalloc: no current CUDA device");
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
      return gw_internal_error(GW_ECUDA, "gw_stage_noalloc: cudaGetSymbolAddress of the scratch array failed");
    g_scratch_addr[dev] = p;
  }
  unsigned char* base = (unsigned char*)g_scratch_addr[dev];
  double* partials = (double*)base;
  unsigned* ticket = (unsigned*)(base + kNoAllocPartialsBytes);
  cudaStream_t st = (cudaStream_t)stream;
  // the scratch keeps the previous call's contents: the ticket must start at 0
  if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), st) != cudaSuccess ||
      cudaMemsetAsync(out + kNoAllocOutError, 0, sizeof(double), st) != cudaSuccess)
    return gw_internal_error(GW_ECUDA, "gw_stage_noalloc: clearing the ticket failed");
  StageParams p = {};
  p.t0 = t0;
  p.tf = tf;
  for (int i = 0; i < 3; i++) {
    p.dep0[i] = dep0[i];
    p.depf[i] = depf[i];
    p.span[i] = depf[i] - dep0[i];
  }
  p.nfru_scale = nfru_scale;
  p.pca_scale = 1.0;  // the reference PCa: this path runs the FP64 one-thread-per-FRU kernel only
  p.epoch = kNoHoldEpoch;
  p.flags = kFlagAdvance;
  const int nblocks = (nfru + kStageThreads - 1) / kStageThreads;
  fru_stage_noalloc_kernel<<<nblocks, kStageThreads, 0, st>>>(nfru, stride, frus, chan, mti, mt, p, partials, ticket,
                                                              out);
  if (cudaGetLastError() != cudaSuccess) return gw_internal_error(GW_ECUDA, "gw_stage_noalloc: launch failed");
  return GW_OK;
}
