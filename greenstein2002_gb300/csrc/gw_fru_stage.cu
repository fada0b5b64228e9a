// FP64 FRU stage kernel: advance every release unit of one cell over one
// Dormand-Prince stage interval and reduce the fluxes the global ODE needs.
//
// Mapping: one thread per FRU (a warp = a group of 32 FRUs).  GB300's FP64
// rate is ~1/64 of FP32, so FP64 work is the bound and a thread-per-FRU layout
// keeps every FP64 lane busy with its own FRU instead of replicating per-FRU
// scalar work across a warp.  FRU state is SoA in HBM (coalesced per warp);
// each FRU's MT19937 words are one 2560-B row that stays L2-resident (a
// 12,500-FRU cell holds 32 MB of MT state, well inside the 129 MB L2).
//
// Reference: simfru_local.c:32-278 (substep loop), fru_rates_local.c:30-798
// (rates; inlined in gw_fru_model.cuh), calc_fru_flux_local.c:28-77 and
// mpi_master.c:401-468 (flux sums and currents), mpi_slave.c:150-226
// (save/resume of FRU + RNG state for rejected steps).
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_fru_model.cuh"
#include "gw_kernels.h"

#include "gw_fru_core.cuh"

namespace gw {

// Flux numerators of the cell, summed in exactly the order of the
// cleft-parallel kernels (gw_fru_cleft.cuh), so every stage kernel gives the
// same bits: per 8-FRU group and cleft a fixed tree over the FRUs
// ((x0+x4)+(x2+x6))+((x1+x5)+(x3+x7)), then (S0+S2)+(S1+S3) over the clefts,
// then the lane-strided last-warp pass over the groups.
__device__ __forceinline__ double group8_sum(double x) {
  x += __shfl_down_sync(0xffffffffu, x, 4);
  x += __shfl_down_sync(0xffffffffu, x, 2);
  x += __shfl_down_sync(0xffffffffu, x, 1);
  return x;  // valid in lanes 0, 8, 16, 24
}

__global__ void __launch_bounds__(kStageThreads) fru_stage_kernel(DevState s, StageParams p) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double x[kClefts][5];
#pragma unroll
  for (int c = 0; c < kClefts; c++)
#pragma unroll
    for (int k = 0; k < 5; k++) x[c][k] = 0.0;
  uint32_t nsub = 0;
  bool overflow = false;
  if (f < s.nfru) {
    const size_t nf = (size_t)s.stride;
    double y[5];
    uint32_t w[kClefts];
    int mti;
    MtRef rng;
    rng.m = s.mt + (size_t)f * kMtStride;
    rng.hold = s.mt_hold + (size_t)f * kMtStride;
    rng.hold_epoch = s.hold_epoch + f;
    rng.epoch = p.epoch;
    if (p.flags & kFlagResume) {
      // mpi_slave.c:150-184: back to the saved FRU and RNG state
#pragma unroll
      for (int i = 0; i < 5; i++) y[i] = s.frus_s[i * nf + f];
#pragma unroll
      for (int c = 0; c < kClefts; c++) w[c] = s.chan_s[c * nf + f];
      mti = s.mti_s[f];
      if (*rng.hold_epoch == p.epoch)
        for (int k = 0; k < kMtN; k++) rng.m[k] = rng.hold[k];
    } else {
#pragma unroll
      for (int i = 0; i < 5; i++) y[i] = s.frus[i * nf + f];
#pragma unroll
      for (int c = 0; c < kClefts; c++) w[c] = s.chan[c * nf + f];
      mti = s.mti[f];
    }
    if (p.flags & kFlagSave) {
      // mpi_slave.c:192-226: snapshot; the MT words are protected lazily by
      // copy-on-twist under the new epoch
#pragma unroll
      for (int i = 0; i < 5; i++) s.frus_s[i * nf + f] = y[i];
#pragma unroll
      for (int c = 0; c < kClefts; c++) s.chan_s[c * nf + f] = w[c];
      s.mti_s[f] = mti;
    }
    rng.mti = mti;
    if (p.flags & kFlagAdvance) advance_fru(p, y, w, rng, nsub, overflow);
    if (overflow) s.out[kOutError] = 1.0;
#pragma unroll
    for (int i = 0; i < 5; i++) s.frus[i * nf + f] = y[i];
#pragma unroll
    for (int c = 0; c < kClefts; c++) s.chan[c * nf + f] = w[c];
    s.mti[f] = rng.mti;
    // flux numerators of this FRU's clefts (calc_fru_flux_local.c:45-70)
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      x[c][0] = y[c + 1];
      if (lcc_open(w[c])) {
        x[c][2] = y[c + 1];
        x[c][3] = 1.0;
      }
      if (cl_of(w[c]) == 2) x[c][4] = 1.0;
    }
    x[0][1] = y[0];
  }
  if (s.substeps) {
    // substep counter (workload accounting): warp-aggregated atomic
    unsigned long long c = nsub;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(s.substeps, c);
  }
  double v[5];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    const double s0 = group8_sum(x[0][k]), s1 = group8_sum(x[1][k]);
    const double s2 = group8_sum(x[2][k]), s3 = group8_sum(x[3][k]);
    v[k] = (s0 + s2) + (s1 + s3);
  }
  // lanes 0, 8, 16, 24 hold the totals of their 8-FRU groups
  const int lane = threadIdx.x & 31;
  const int ngroups = (s.nfru + 7) >> 3, grp0 = (blockIdx.x * blockDim.x) >> 3;
  const int mine = min(4, ngroups - grp0);  // groups of this warp that hold FRUs
  unsigned last = 0u;
  if ((lane & 7) == 0 && (lane >> 3) < mine) {
#pragma unroll
    for (int k = 0; k < 5; k++) s.partials[(grp0 + (lane >> 3)) * 5 + k] = v[k];
  }
  __syncwarp();
  if (lane == 0) {
    __threadfence();
    last = (atomicAdd(s.ticket, (unsigned)mine) == (unsigned)(ngroups - mine)) ? 1u : 0u;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  double tot[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = lane; b < ngroups; b += 32)
#pragma unroll
    for (int k = 0; k < 5; k++) tot[k] += __ldcg(&s.partials[b * 5 + k]);
#pragma unroll
  for (int k = 0; k < 5; k++)
    for (int o = 16; o > 0; o >>= 1) tot[k] += __shfl_down_sync(0xffffffffu, tot[k], o);
  if (lane == 0) {
    *s.ticket = 0u;
    double cur[4];
    currents_from_sums(s.nfru, p.nfru_scale, p.depf, tot, cur);
#pragma unroll
    for (int k = 0; k < 5; k++) s.out[k] = tot[k];
#pragma unroll
    for (int k = 0; k < 4; k++) s.out[5 + k] = cur[k];
  }
}

// Output-cadence sums of calc_fru_avg_local.c:27-105 (11 values).
__global__ void __launch_bounds__(kStageThreads) fru_avg_kernel(DevState s) {
  __shared__ double smem[32 * 11];
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double v[11];
#pragma unroll
  for (int k = 0; k < 11; k++) v[k] = 0.0;
  if (f < s.nfru) {
    const size_t nf = (size_t)s.stride;
    const double jsr = s.frus[f];
    v[1] = jsr;
    v[6] = jsr * (1.0 + CSQNtot / (KmCSQN + jsr));
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      const double ss = s.frus[(c + 1) * nf + f];
      const uint32_t w = s.chan[c * nf + f];
      int no = 0, ready = 0;
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        const int r = ryr_of(w, i);
        no += ryr_open(r);
        ready += (r == 1 || r == 2);
      }
      v[0] += ss;
      v[5] += ss * (1.0 + BSRtot / (KBSR + ss) + BSLtot / (KBSL + ss));
      v[2] += JRyRmax * ((double)no) * (jsr - ss);
      v[3] += (double)no;
      v[4] += (double)ready;
      if (lcc_of(w) <= 6) v[7] += 1.0;
      if (vdi_of(w) == 2) v[8] += 1.0;
      if (lcc_open(w)) v[9] += 1.0;
      if (cl_of(w) == 2) v[10] += 1.0;
    }
  }
  block_reduce<11>(v, smem);
  double tot[11];
  if (grid_finish<11>(v, s.partials, s.ticket, smem, tot))
#pragma unroll
    for (int k = 0; k < 11; k++) s.out[16 + k] = tot[k];
}

// Reference-order sums (the parity mode of gw_set_sum_order): the flux
// numerators added one FRU and one cleft after another, as
// calc_fru_flux_local.c:44-70 does, then the currents of
// mpi_master.c:447-468.  A sequential FP64 sum has exactly one rounding
// order, so each sum is one thread's dependent chain; the block stages the
// stored FRU states in shared memory in coalesced chunks and three warps (on
// three SM sub-partitions) run the three chains side by side: the CaSS sum,
// the CaJSR sum, and the open-LCC CaSS sum with the two counts (integers,
// exact).  About 4 dependent FP64 additions per FRU, so this mode is for
// parity runs of small cells.  Runs after the stage launch and overwrites
// out[0..8].
constexpr int kSeqThreads = 128, kSeqChunk = 512;
__global__ void __launch_bounds__(kSeqThreads) fru_flux_seq_kernel(DevState s, StageParams p) {
  __shared__ double sf[5][kSeqChunk];
  __shared__ uint32_t sw[kClefts][kSeqChunk];
  __shared__ double res[5];
  const size_t nf = (size_t)s.stride;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double acc = 0.0;  // warp 0: sum CaSS; warp 1: sum CaJSR; warp 2: sum CaSS of open LCCs
  int oca = 0, ncl = 0;
  for (int base = 0; base < s.nfru; base += kSeqChunk) {
    const int cnt = min(kSeqChunk, s.nfru - base);
    for (int i = threadIdx.x; i < 5 * cnt; i += kSeqThreads) sf[i / cnt][i % cnt] = s.frus[(i / cnt) * nf + base + i % cnt];
    for (int i = threadIdx.x; i < kClefts * cnt; i += kSeqThreads)
      sw[i / cnt][i % cnt] = s.chan[(i / cnt) * nf + base + i % cnt];
    __syncthreads();
    if (lane == 0 && warp == 0) {
      for (int j = 0; j < cnt; j++)
#pragma unroll
        for (int c = 0; c < kClefts; c++) acc += sf[c + 1][j];
    } else if (lane == 0 && warp == 1) {
      for (int j = 0; j < cnt; j++) acc += sf[0][j];
    } else if (lane == 0 && warp == 2) {
      for (int j = 0; j < cnt; j++)
#pragma unroll
        for (int c = 0; c < kClefts; c++) {
          const uint32_t w = sw[c][j];
          if (lcc_open(w)) {
            acc = acc + sf[c + 1][j];
            oca++;
          }
          if (cl_of(w) == 2) ncl++;
        }
    }
    __syncthreads();
  }
  if (lane == 0 && warp < 3) {
    res[warp == 0 ? 0 : warp == 1 ? 1 : 2] = acc;
    if (warp == 2) {
      res[3] = (double)oca;
      res[4] = (double)ncl;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double tot[5] = {res[0], res[1], res[2], res[3], res[4]};
    double cur[4];
    currents_from_sums(s.nfru, p.nfru_scale, p.depf, tot, cur);
    cur[2] = cur[2] * p.pca_scale;
#pragma unroll
    for (int k = 0; k < 5; k++) s.out[k] = tot[k];
#pragma unroll
    for (int k = 0; k < 4; k++) s.out[5 + k] = cur[k];
  }
}

// The 11 output sums in the order of calc_fru_avg_local.c:50-91 (one thread,
// the parity mode's counterpart of fru_avg_kernel).
__global__ void __launch_bounds__(32) fru_avg_seq_kernel(DevState s) {
  if (threadIdx.x != 0) return;
  const size_t nf = (size_t)s.stride;
  double v[11];
#pragma unroll
  for (int k = 0; k < 11; k++) v[k] = 0.0;
  int ready = 0;
  for (int f = 0; f < s.nfru; f++) {
    const double jsr = s.frus[f];
    v[1] = v[1] + jsr;
    v[6] = v[6] + jsr * (1.0 + CSQNtot / (KmCSQN + jsr));
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      const double ss = s.frus[(c + 1) * nf + f];
      const uint32_t w = s.chan[c * nf + f];
      v[0] = v[0] + ss;
      v[5] = v[5] + ss * (1.0 + BSRtot / (KBSR + ss) + BSLtot / (KBSL + ss));
      int no = 0;
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        const int r = ryr_of(w, i);
        no += ryr_open(r);
        ready += (r == 1 || r == 2);
      }
      v[2] = v[2] + JRyRmax * ((double)no) * (jsr - ss);
      v[3] = v[3] + (double)no;
      if (lcc_of(w) <= 6) v[7] = v[7] + 1.0;
      if (vdi_of(w) == 2) v[8] = v[8] + 1.0;
      if (lcc_open(w)) v[9] = v[9] + 1.0;
      if (cl_of(w) == 2) v[10] = v[10] + 1.0;
    }
  }
  v[4] = (double)ready;
#pragma unroll
  for (int k = 0; k < 11; k++) s.out[16 + k] = v[k];
}

// Knuth initialisation of every FRU's MT19937 state (mt19937_local.c:76-92),
// seeded either by base + j or by the formula of initialize_ran.c:30-34.
__global__ void fru_seed_kernel(DevState s, int scheme, uint32_t base) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= s.nfru) return;
  uint32_t seed;
  if (scheme == kSeedReference) {
    // a_j = 12350232 + 23*(0+1+..+j); seed = |a_j + 4093*j*j| + 1 in 32-bit
    // two's-complement arithmetic
    const uint32_t j = (uint32_t)f;
    const uint32_t tri = (uint32_t)(((uint64_t)j * (uint64_t)(j + 1)) / 2u);
    const uint32_t a = 12350232u + 23u * tri;
    int32_t t = (int32_t)(a + (4093u * j) * j);
    if (t < 0) t = (int32_t)(0u - (uint32_t)t);
    seed = (uint32_t)t + 1u;
  } else {
    seed = base + (uint32_t)f;
  }
  uint32_t* m = s.mt + (size_t)f * kMtStride;
  uint32_t x = seed;
  m[0] = x;
  for (uint32_t i = 1; i < kMtN; i++) {
    x = 1812433253u * (x ^ (x >> 30)) + i;
    m[i] = x;
  }
  s.mti[f] = kMtN;
  s.hold_epoch[f] = 0xffffffffu;
}

}  // namespace gw

// ---- launchers (C++ linkage, used by gw_abi.cu) -------------------------------
namespace gw {
cudaError_t launch_stage(const DevState& s, const StageParams& p, cudaStream_t st) {
  fru_stage_kernel<<<s.nblocks, kStageThreads, 0, st>>>(s, p);
  return cudaGetLastError();
}
cudaError_t launch_avg(const DevState& s, cudaStream_t st) {
  fru_avg_kernel<<<s.nblocks, kStageThreads, 0, st>>>(s);
  return cudaGetLastError();
}
cudaError_t launch_flux_seq(const DevState& s, const StageParams& p, cudaStream_t st) {
  fru_flux_seq_kernel<<<1, kSeqThreads, 0, st>>>(s, p);
  return cudaGetLastError();
}
cudaError_t launch_avg_seq(const DevState& s, cudaStream_t st) {
  fru_avg_seq_kernel<<<1, 32, 0, st>>>(s);
  return cudaGetLastError();
}
cudaError_t launch_seed(const DevState& s, int scheme, uint32_t base, cudaStream_t st) {
  fru_seed_kernel<<<s.nblocks, kStageThreads, 0, st>>>(s, scheme, base);
  return cudaGetLastError();
}
}  // namespace gw
