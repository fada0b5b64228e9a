// Device building blocks of the FRU stage: the substep loop of one FRU and
// the deterministic flux reduction.  Shared by the FRU stage kernels.
//
// Reference: simfru_local.c:32-278, calc_fru_flux_local.c:28-77,
// mpi_master.c:447-468.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_fru_model.cuh"
#include "gw_kernels.h"

namespace gw {

// Deterministic block reduction of NV doubles: warp shuffles, then warps in
// index order.  Result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_reduce(double v[NV], double* smem /* [32][NV] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) smem[warp * NV + k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double s = smem[k];
      for (int w = 1; w < nwarp; w++) s += smem[w * NV + k];
      v[k] = s;
    }
  }
  __syncthreads();
}

// Last-block pass: sum the per-block partials in a fixed order, so the result
// does not depend on which block finished last.  Returns true in thread 0 of
// the last block, with the totals in tot[].
template <int NV>
__device__ __forceinline__ bool grid_finish(const double v[NV], double* partials, unsigned* ticket, double* smem,
                                            double tot[NV]) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) partials[blockIdx.x * NV + k] = v[k];
    __threadfence();
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) s[k] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; k++) s[k] += __ldcg(&partials[b * NV + k]);
  block_reduce<NV>(s, smem);
  if (threadIdx.x == 0) {
    *ticket = 0u;
#pragma unroll
    for (int k = 0; k < NV; k++) tot[k] = s[k];
  }
  return threadIdx.x == 0;
}

// Flux numerators -> (Jxfer, Jtr, ICa, Ito2): mpi_master.c:447-468.
static __device__ void currents_from_sums(int nfru, double scale, const double dep[3], const double num[5], double out[4]) {
  const double V = dep[0], Cai = dep[1], CaNSR = dep[2];
  const double VFRT = V / RT_over_F, VFsqRT = (1000.0 * Faraday) * VFRT;
  const double e1 = exp(VFRT), e2 = e1 * e1;
  double ica, ito2;
  if (fabs(V) < 1.e-6) {
    const double icanum = num[2] - num[3] * Cao * 0.341;
    ica = PCa * 2.0 * 1000.0 * Faraday * icanum;
    ica = ica / Acap;
    ito2 = num[4] * PCl * 1000.0 * Faraday * (Clo - Cli);
    ito2 = ito2 / Acap;
  } else {
    const double icanum = num[2] * e2 - num[3] * Cao * 0.341;
    ica = PCa * 4.0 * VFsqRT * icanum / (e2 - 1.0);
    ica = ica / Acap;
    ito2 = num[4] * PCl * VFsqRT * (Cli - Clo * e1) / (1.0 - e1);
    ito2 = ito2 / Acap;
  }
  const double jtr = (((double)nfru) * CaNSR - num[1]) / tautr;
  const double jxfer = (num[0] - ((double)nfru * (double)kClefts) * Cai) / tauxfer;
  out[0] = scale * jxfer;
  out[1] = scale * jtr;
  out[2] = scale * ica;
  out[3] = scale * ito2;
}

// Categorical selection of simfru_local.c:217-226 for a channel that has left
// its state (u > 1 - dt*total): walk the cumulative probabilities.
__device__ __forceinline__ int pick_dest(const double r[4], const int d[4], int len, double dt, double u) {
  double acc = 1.0 - dt * r[0];
  int n = 1;
  acc += dt * r[1];
  while (u > acc && n + 1 < len) {
    n++;
    acc += dt * r[n];
  }
  return d[n];
}

// Upper bound on substeps of one FRU in one stage.  Valid states need far
// fewer (dt >= 0.1 / max exit rate, and rates are bounded); corrupted input
// (NaN or huge concentrations) stops here with an error flag instead of
// looping without end.
constexpr uint32_t kMaxSubsteps = 1u << 22;

// One FRU over [t0, tf]: simfru_local.c:83-277.
__device__ __forceinline__ void advance_fru(const StageParams& p, double y[5], uint32_t w[kClefts], MtRef& rng,
                                            uint32_t& nsub, bool& overflow) {
  double dep[3], lopen[kClefts], R0[32];
  int nopen[kClefts];
#pragma unroll
  for (int i = 0; i < 3; i++) dep[i] = p.dep0[i];
#pragma unroll
  for (int c = 0; c < kClefts; c++) {
    lopen[c] = lcc_open(w[c]) ? 1.0 : 0.0;
    nopen[c] = ryr_open_count(w[c]);
  }
  const double interval = p.tf - p.t0;
  double t = p.t0;
  while (t < p.tf) {
    if (nsub >= kMaxSubsteps) {
      overflow = true;
      break;
    }
    // ---- exit rates at the substep start (fru_rates_local.c:126-777) ----
    const LccBasis lb = lcc_basis(dep[0]);
    const double nu = 1.0;
    const double yinf = nu * (0.4 / (1.0 + exp((dep[0] + 12.5) / 5.0)) + (1.0 - 0.4));
    const double tau = 60.0 + 340.0 / (1.0 + exp((dep[0] + 30.0) / 12.0));
    const double vdi_open_rate = (1.0 - yinf) / tau, vdi_closed_rate = yinf / tau;
    double cass0[kClefts];
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      cass0[c] = y[c + 1];
      R0[8 * c + 0] = lcc_total(lcc_of(w[c]), lb, gammacf * y[c + 1]);
      R0[8 * c + 1] = (vdi_of(w[c]) == 2) ? vdi_open_rate : vdi_closed_rate;
    }
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      const RyrK k = ryr_constants(y[c + 1]);
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        const int s = ryr_resolve(ryr_of(w[c], i), k, rng);
        w[c] = set_field(w[c], 8 + 4 * i, s);
        R0[8 * c + 2 + i] = ryr_total(s, k);
      }
      R0[8 * c + 7] = (cl_of(w[c]) == 1) ? kfIto2 * y[c + 1] : kbIto2;
    }
    double mx = 0.0;
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      mx = dmax(mx, R0[8 * c + 0]);
      mx = dmax(mx, R0[8 * c + 1]);
      mx = dmax(mx, R0[8 * c + 7]);
#pragma unroll
      for (int i = 0; i < kRyR; i++) mx = dmax(mx, R0[8 * c + 2 + i]);
    }
    // ---- substep size (simfru_local.c:135-146) ----
    double dt = dmin(0.1 / mx, 10.001e-3);
    double cmax = 0.e-3;
#pragma unroll
    for (int c = 0; c < kClefts; c++) cmax = dmax(cmax, y[c + 1]);
    if (cmax > 1.5e-3) dt = dmin(dt, 5.001e-3);
    dt = dmin(dt, p.tf - t);
    // ---- Heun step of the local Ca ODE with pre-transition flags (:149-173) ----
    double k1[5], y1[5], dF[5];
    fcn_fru(y, dep, lopen, nopen, dF);
#pragma unroll
    for (int i = 0; i < 5; i++) {
      k1[i] = dt * dF[i];
      y1[i] = y[i] + k1[i];
    }
    t = t + dt;
#pragma unroll
    for (int i = 0; i < 3; i++) dep[i] = p.dep0[i] + (t - p.t0) / interval * p.span[i];
    fcn_fru(y1, dep, lopen, nopen, dF);
#pragma unroll
    for (int i = 0; i < 5; i++) y[i] = y[i] + (k1[i] + dt * dF[i]) / 2.0;
    // ---- 32 uniforms and transitions (:211-276) ----
#pragma unroll
    for (int c = 0; c < kClefts; c++) {
      bool moved = false;
      // LCC
      {
        const double u = rng.next();
        if (u > 1.0 - dt * R0[8 * c]) {
          double r[4];
          int d[4];
          const int len = lcc_row(lcc_of(w[c]), lb, gammacf * cass0[c], r, d);
          w[c] = set_field(w[c], 0, pick_dest(r, d, len, dt, u));
        }
      }
      // voltage-dependent inactivation gate
      {
        const double u = rng.next();
        if (u >= 1.0 - dt * R0[8 * c + 1]) w[c] = set_field(w[c], 4, 3 - vdi_of(w[c]));
      }
      // RyRs
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        const double u = rng.next();
        if (u > 1.0 - dt * R0[8 * c + 2 + i]) {
          const RyrK k = ryr_constants(cass0[c]);
          double r[4];
          int d[4];
          const int len = ryr_row(ryr_of(w[c], i), k, r, d);
          w[c] = set_field(w[c], 8 + 4 * i, pick_dest(r, d, len, dt, u));
          moved = true;
        }
      }
      // Ca-activated Cl channel
      {
        const double u = rng.next();
        if (u >= 1.0 - dt * R0[8 * c + 7]) w[c] = set_field(w[c], 28, 3 - cl_of(w[c]));
      }
      lopen[c] = lcc_open(w[c]) ? 1.0 : 0.0;
      if (moved) nopen[c] = ryr_open_count(w[c]);
    }
    nsub++;
  }
}

}  // namespace gw
