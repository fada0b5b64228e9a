// Device-side Dormand-Prince 5(4) integrator of one cell's 37 global states
// (rk_pd54m.c:29-345), shared by the device-resident runners: the graph of
// rounds (gw_devdp.cu) and the persistent multi-cell kernel (gw_persist.cu).
//
// A DpCell holds the integrator's state (y, k1..k5, the trial state,
// start/step/ostep, the accept/reject state) and the parameters of the cell's
// next FRU launch; dp_after advances it after one FRU launch exactly as the
// host integrator (gw_dp.c) does, operation for operation (compiled with
// -fmad=false), and sets up the next launch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_cell_model.h"
#include "gw_kernels.h"

namespace gw {

enum : int { kPhFlux = 0, kPhS2 = 1, kPhS3 = 2, kPhS4 = 3, kPhS5 = 4, kPhS6 = 5 };

// the integrator's min/max (ties return the first argument, as gw_dp.c)
__device__ __forceinline__ double fmin_ref(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double fmax_ref(double a, double b) { return a < b ? b : a; }

struct DpCell {
  double y[GW_NSTATE], F1[GW_NSTATE], k[5][GW_NSTATE], y1[GW_NSTATE], cur[GW_NCUR];
  double tnow, start, tstep, step, ostep, oldstep;
  double dep0[3];
  gw_settings set;
  StageParams sp;      // the cell's next FRU launch
  int phase, success, keepc, pending, steps_left, step_index, done, final_avg, err;
  uint32_t epoch;
  double* tr_states;   // [n_steps][37] (device, may be null)
  double* tr_other;    // [n_steps][12]
  double* tr_cur;      // [n_steps][24]
  int nfru;
  gw_tx tx;                // the transcendental terms of the last fcn (warp integrator)
  double y5[GW_NSTATE];    // the fifth-order trial state after stage 6 (warp integrator)
};


__device__ __forceinline__ void dep_of(const double* y, double d[3]) {
  d[0] = y[GW_V];
  d[1] = y[GW_Cai];
  d[2] = y[GW_CaNSR];
}

static __device__ inline void set_launch(DpCell& c, double t0, double tf, const double dep0[3], const double depf[3], int advance) {
  StageParams& p = c.sp;
  p.t0 = t0;
  p.tf = tf;
  for (int i = 0; i < 3; i++) {
    p.dep0[i] = dep0[i];
    p.depf[i] = depf[i];
    p.span[i] = depf[i] - dep0[i];
  }
  p.epoch = c.epoch;
  p.flags = c.pending | (advance ? kFlagAdvance : 0);
  c.pending = 0;
}

// flux-only launch at an attempt's start (gw_flux), optionally with the
// output averages of the state the previous output step ended in
static __device__ inline void launch_flux(DpCell& c, bool avg) {
  double d[3];
  dep_of(c.y, d);
  set_launch(c, 0.0, 0.0, d, d, 0);
  if (avg) c.sp.flags |= kFlagAvg;
}

// stage 2 (node 1/5) from F1 and the current step (rk_pd54m.c:121-127)
static __device__ inline void launch_stage2(DpCell& c) {
  double* k1 = c.k[0];
  for (int i = 0; i < GW_NSTATE; i++) {
    k1[i] = c.step * c.F1[i];
    c.y1[i] = c.y[i] + k1[i] / 5.0;
  }
  double depf[3];
  dep_of(c.y, c.dep0);
  dep_of(c.y1, depf);
  set_launch(c, c.start, c.start + c.step / 5.0, c.dep0, depf, 1);
  c.phase = kPhS2;
}

// the start of an output step (gw_rk54pd's preamble)
static __device__ inline void begin_output_step(DpCell& c) {
  c.tstep = c.tnow + c.set.time_step;
  double step = fmin_ref(c.oldstep, c.tstep - c.tnow);
  step = fmin_ref(c.set.step_max, step);
  c.step = step;
  c.ostep = step;
  c.start = c.tnow;
  c.success = 1;
  c.keepc = 1;
}

// The integrator after one FRU launch of the cell; J = (Jxfer, Jtr, ICa,
// Ito2) at the launch's end point; avg = the output-average sums when the
// launch carried them.
static __device__ __noinline__ void dp_after(DpCell& c, const double J[4], const double* avg) {
  double F[GW_NSTATE], dummy[GW_NCUR];
  const double step = c.step, start = c.start;
  double* k1 = c.k[0];
  double* k2 = c.k[1];
  double* k3 = c.k[2];
  double* k4 = c.k[3];
  double* k5 = c.k[4];
  if (c.phase == kPhFlux) {
    if (avg && c.step_index > 0 && c.tr_other)
      gw_otherstates(avg, c.nfru, 12500.0 / (double)c.nfru, c.y, c.tr_other + (size_t)(c.step_index - 1) * GW_NOTHER);
    if (c.final_avg) {
      c.done = 1;
      return;
    }
    gw_fcn(start, c.y, c.F1, c.cur, c.keepc, J[0], J[1], J[2], J[3], &c.set);
    c.keepc = 0;
    c.epoch++;  // gw_save: a new snapshot epoch, folded into the next launch
    c.pending = kFlagSave;
    launch_stage2(c);
    return;
  }
  double depf[3];
  switch (c.phase) {
    case kPhS2:
      gw_fcn(start + step / 5.0, c.y1, F, dummy, 0, J[0], J[1], J[2], J[3], &c.set);
      for (int i = 0; i < GW_NSTATE; i++) {
        k2[i] = step * F[i];
        c.y1[i] = c.y[i] + (3.0 / 40.0 * k1[i] + 9.0 / 40.0 * k2[i]);
      }
      dep_of(c.y1, depf);
      set_launch(c, start + step / 5.0, start + step * 3.0 / 10.0, c.dep0, depf, 1);
      c.phase = kPhS3;
      return;
    case kPhS3:
      gw_fcn(start + step * 3.0 / 10.0, c.y1, F, dummy, 0, J[0], J[1], J[2], J[3], &c.set);
      for (int i = 0; i < GW_NSTATE; i++) {
        k3[i] = step * F[i];
        c.y1[i] = c.y[i] + (3.0 / 10.0 * k1[i] - 9.0 / 10.0 * k2[i] + 6.0 / 5.0 * k3[i]);
      }
      dep_of(c.y1, depf);
      set_launch(c, start + step * 3.0 / 10.0, start + step * 3.0 / 5.0, c.dep0, depf, 1);
      c.phase = kPhS4;
      return;
    case kPhS4:
      gw_fcn(start + step * 3.0 / 5.0, c.y1, F, dummy, 0, J[0], J[1], J[2], J[3], &c.set);
      for (int i = 0; i < GW_NSTATE; i++) {
        k4[i] = F[i] * step;
        c.y1[i] = c.y[i] + 226.0 / 729.0 * k1[i] - 25.0 / 27.0 * k2[i] + 880.0 / 729.0 * k3[i] +
                  55.0 / 729.0 * k4[i];
      }
      dep_of(c.y1, depf);
      set_launch(c, start + step * 3.0 / 5.0, start + step * 2.0 / 3.0, c.dep0, depf, 1);
      c.phase = kPhS5;
      return;
    case kPhS5:
      gw_fcn(start + step * 2.0 / 3.0, c.y1, F, dummy, 0, J[0], J[1], J[2], J[3], &c.set);
      for (int i = 0; i < GW_NSTATE; i++) {
        k5[i] = step * F[i];
        c.y1[i] = c.y[i] - 181.0 / 270.0 * k1[i] + 5.0 / 2.0 * k2[i] - 266.0 / 297.0 * k3[i] -
                  91.0 / 27.0 * k4[i] + 189.0 / 55.0 * k5[i];
      }
      dep_of(c.y1, depf);
      set_launch(c, start + step * 2.0 / 3.0, start + step, c.dep0, depf, 1);
      c.phase = kPhS6;
      return;
    default:
      break;
  }
  // after stage 6: error estimate and step control (rk_pd54m.c:215-333)
  gw_fcn(start + step, c.y1, F, dummy, 0, J[0], J[1], J[2], J[3], &c.set);
  const double huge_number = 1e99, min_tolvalue = 1.e-10;
  double tr = 0.0, y5[GW_NSTATE];
  for (int i = 0; i < GW_NSTATE; i++) {
    const double k6 = step * F[i];
    y5[i] = c.y[i] + 31.0 / 540.0 * k1[i] + 190.0 / 297.0 * k3[i] - 145.0 / 108.0 * k4[i] + 351.0 / 220.0 * k5[i] +
            1.0 / 20.0 * k6;
    const double ym = c.y[i] + 19.0 / 216.0 * k1[i] + 1000.0 / 2079.0 * k3[i] - 125.0 / 216.0 * k4[i] +
                      81.0 / 88.0 * k5[i] + 5.0 / 56.0 * k6;
    const double err = fabs((ym - y5[i]) * 0.2 * gw_errweight(i));
    if (err < huge_number) tr = fmax_ref(err, tr);
    else tr = huge_number;
  }
  const gw_settings& P = c.set;
  bool finished_output = false;
  if (tr < P.tolrk || step <= P.step_min) {
    // an accepted state that is not finite would only be accepted again at
    // the minimum step, forever: the cell stops with an error instead
    bool finite = true;
    for (int i = 0; i < GW_NSTATE; i++) finite = finite && isfinite(y5[i]);
    if (!finite) {
      c.err = 2;
      return;
    }
  }
  if (tr < P.tolrk) {
    for (int i = 0; i < GW_NSTATE; i++) {
      if (fabs(y5[i]) < min_tolvalue) y5[i] = 0.0;
      c.y[i] = y5[i];
    }
    c.start = start + step;
    c.success = 1;
    if (c.start >= c.tstep) {
      finished_output = true;
    } else {
      double nstep = fmin_ref(0.85 * step * pow(P.tolrk / tr, 0.2), 4.0 * step);
      c.ostep = nstep;
      double tts = P.shift - fmod(c.start, P.period);
      if (tts < 0.0) tts = tts + P.period;
      if (tts < nstep) nstep = fmax_ref(P.step_min, tts - 0.5 * P.step_min);
      c.step = nstep;
    }
  } else if (step <= P.step_min) {
    // forced accept at the minimum step
    for (int i = 0; i < GW_NSTATE; i++) {
      if (fabs(y5[i]) < min_tolvalue) y5[i] = 0.0;
      c.y[i] = y5[i];
    }
    c.start = start + step;
    c.success = 1;
    if (c.start >= c.tstep) {
      finished_output = true;
    } else {
      c.step = P.step_min;
    }
    c.ostep = c.step;
  } else {
    // reject: roll the FRUs back and retry from stage 2 (no new flux/save)
    double nstep = 0.85 * step * pow(P.tolrk / tr, 0.2);
    double tts = P.shift - fmod(start, P.period);
    if (tts < 0.0) tts = tts + P.period;
    if (tts < nstep) nstep = fmax_ref(P.step_min, tts - 0.5 * P.step_min);
    c.success = 0;
    c.pending = kFlagResume;
    nstep = fmin_ref(P.step_max, fmax_ref(P.step_min, nstep));
    c.step = fmin_ref(nstep, c.tstep - c.start);
    c.oldstep = c.ostep;
    launch_stage2(c);
    return;
  }
  if (!finished_output && !(tr < P.tolrk)) {
    // the forced-accept branch clamps like a rejection (rk_pd54m.c:329-331)
    c.step = fmin_ref(P.step_max, fmax_ref(P.step_min, c.step));
    c.step = fmin_ref(c.step, c.tstep - c.start);
  }
  c.oldstep = c.ostep;
  if (!finished_output) {
    launch_flux(c, false);
    c.phase = kPhFlux;
    return;
  }
  // an output step is complete (gw_run): record it and start the next one
  const int k = c.step_index;
  if (c.tr_states)
    for (int i = 0; i < GW_NSTATE; i++) c.tr_states[(size_t)k * GW_NSTATE + i] = c.y[i];
  if (c.tr_cur)
    for (int i = 0; i < GW_NCUR; i++) c.tr_cur[(size_t)k * GW_NCUR + i] = c.cur[i];
  c.step_index = k + 1;
  c.steps_left--;
  c.tnow = c.tnow + P.time_step;
  if (c.steps_left <= 0) c.final_avg = 1;
  else begin_output_step(c);
  launch_flux(c, c.tr_other != nullptr || c.final_avg);
  c.phase = kPhFlux;
  if (c.final_avg && !c.tr_other) c.done = 1;
}

// ---- the same integrator on a whole warp --------------------------------------------
// dp_after_warp does what dp_after does, with every lane of a warp taking
// part: the scalar decisions are computed on every lane alike (the FP64
// pipe issues one warp instruction for one lane or for 32), the 37-element
// vector operations are split over the lanes (lane l owns states l and
// l + 32), the exponentials of fcn are evaluated one per lane, and each
// value is written to the DpCell by one lane only.  Each state's arithmetic
// is dp_after's, operation for operation, and the error norm is the same
// maximum, so the results are the same bits.

// fcn's transcendental terms for `state` at `time`: lane k evaluates
// exponent k, lanes 0-1 the last two exponents, 2-5 the logs, 6-11 the pows
// (the functions of gw_tx_fill), lane 0 then K1_inf's exponential.
__device__ __forceinline__ void tx_fill_warp(const double time, const double* state, const gw_protocol* P, gw_tx* tx,
                                             int lane) {
  double Istim;
  const double V = gw_fcn_voltage(time, state, P, &Istim);
  tx->x[lane] = exp(gw_x_arg(lane, V));
  if (lane < GW_NX - 32) {
    tx->x[32 + lane] = exp(gw_x_arg(32 + lane, V));
  } else if (lane < GW_NX - 32 + 4) {
    tx->lg[lane - (GW_NX - 32)] = log(gw_lg_arg(lane - (GW_NX - 32), state));
  } else if (lane < GW_NX - 32 + 10) {
    double y;
    const int k = lane - (GW_NX - 32 + 4);
    const double b = gw_pw_arg(k, state, &y);
    tx->pw[k] = pow(b, y);
  }
  __syncwarp();
  if (lane == 0) tx->k1 = exp(gw_k1_arg(V, tx->lg));
  __syncwarp();
}

// fcn of the state y (global, in the DpCell) on every lane: F and cur
// receive the derivatives and (keepc) the currents in each lane's registers;
// fcn's in-place updates of y (mNa below -90 mV, V under a clamp) are
// written back by lane 0.
__device__ __forceinline__ void fcn_warp(DpCell& c, double time, double* y, double* F, double* cur, int keepc,
                                         const double J[4], int lane) {
  double ys[GW_NSTATE];
#pragma unroll
  for (int i = 0; i < GW_NSTATE; i++) ys[i] = y[i];
  tx_fill_warp(time, ys, &c.set, &c.tx, lane);
  gw_fcn_tx(time, ys, F, cur, keepc, J[0], J[1], J[2], J[3], &c.set, &c.tx);
  __syncwarp();
  if (lane == 0) {
    y[GW_mNa] = ys[GW_mNa];
    y[GW_V] = ys[GW_V];
  }
  __syncwarp();
}

// stage 2 (node 1/5) from F1 with the step `step` (launch_stage2)
__device__ __forceinline__ void launch_stage2_warp(DpCell& c, double step, int lane) {
  for (int i = lane; i < GW_NSTATE; i += 32) {
    const double k1 = step * c.F1[i];
    c.k[0][i] = k1;
    c.y1[i] = c.y[i] + k1 / 5.0;
  }
  __syncwarp();
  if (lane == 0) {
    double depf[3];
    dep_of(c.y, c.dep0);
    dep_of(c.y1, depf);
    set_launch(c, c.start, c.start + step / 5.0, c.dep0, depf, 1);
    c.phase = kPhS2;
  }
  __syncwarp();
}

__device__ __forceinline__ double warp_max_ref(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax_ref(__shfl_xor_sync(0xffffffffu, v, o), v);
  return v;
}

static __device__ __noinline__ void dp_after_warp(DpCell& c, const double J[4], const double* avg, int lane) {
  double F[GW_NSTATE], cur[GW_NCUR];
  __syncwarp();
  const double step = c.step, start = c.start;
  const int phase = c.phase;
  double* k1 = c.k[0];
  double* k2 = c.k[1];
  double* k3 = c.k[2];
  double* k4 = c.k[3];
  double* k5 = c.k[4];
  if (phase == kPhFlux) {
    if (lane == 0 && avg && c.step_index > 0 && c.tr_other)
      gw_otherstates(avg, c.nfru, 12500.0 / (double)c.nfru, c.y, c.tr_other + (size_t)(c.step_index - 1) * GW_NOTHER);
    if (c.final_avg) {
      __syncwarp();
      if (lane == 0) c.done = 1;
      __syncwarp();
      return;
    }
    const int keepc = c.keepc;
    fcn_warp(c, start, c.y, F, cur, keepc, J, lane);
    for (int i = lane; i < GW_NSTATE; i += 32) c.F1[i] = F[i];
    if (lane == 0) {
      if (keepc)
        for (int i = 0; i < GW_NCUR; i++) c.cur[i] = cur[i];
      c.keepc = 0;
      c.epoch++;  // gw_save: a new snapshot epoch, folded into the next launch
      c.pending = kFlagSave;
    }
    __syncwarp();
    launch_stage2_warp(c, step, lane);
    return;
  }
  if (phase != kPhS6) {
    double t_node, t_next;
    if (phase == kPhS2) {
      t_node = start + step / 5.0;
      t_next = start + step * 3.0 / 10.0;
    } else if (phase == kPhS3) {
      t_node = start + step * 3.0 / 10.0;
      t_next = start + step * 3.0 / 5.0;
    } else if (phase == kPhS4) {
      t_node = start + step * 3.0 / 5.0;
      t_next = start + step * 2.0 / 3.0;
    } else {
      t_node = start + step * 2.0 / 3.0;
      t_next = start + step;
    }
    fcn_warp(c, t_node, c.y1, F, cur, 0, J, lane);
    for (int i = lane; i < GW_NSTATE; i += 32) {
      if (phase == kPhS2) {
        k2[i] = step * F[i];
        c.y1[i] = c.y[i] + (3.0 / 40.0 * k1[i] + 9.0 / 40.0 * k2[i]);
      } else if (phase == kPhS3) {
        k3[i] = step * F[i];
        c.y1[i] = c.y[i] + (3.0 / 10.0 * k1[i] - 9.0 / 10.0 * k2[i] + 6.0 / 5.0 * k3[i]);
      } else if (phase == kPhS4) {
        k4[i] = F[i] * step;
        c.y1[i] = c.y[i] + 226.0 / 729.0 * k1[i] - 25.0 / 27.0 * k2[i] + 880.0 / 729.0 * k3[i] +
                  55.0 / 729.0 * k4[i];
      } else {
        k5[i] = step * F[i];
        c.y1[i] = c.y[i] - 181.0 / 270.0 * k1[i] + 5.0 / 2.0 * k2[i] - 266.0 / 297.0 * k3[i] -
                  91.0 / 27.0 * k4[i] + 189.0 / 55.0 * k5[i];
      }
    }
    __syncwarp();
    if (lane == 0) {
      double depf[3];
      dep_of(c.y1, depf);
      set_launch(c, t_node, t_next, c.dep0, depf, 1);
      c.phase = phase + 1;
    }
    __syncwarp();
    return;
  }
  // after stage 6: error estimate and step control (rk_pd54m.c:215-333)
  fcn_warp(c, start + step, c.y1, F, cur, 0, J, lane);
  const double huge_number = 1e99, min_tolvalue = 1.e-10;
  double tr = 0.0;
  bool bad = false, finite = true;
  for (int i = lane; i < GW_NSTATE; i += 32) {
    const double k6 = step * F[i];
    const double y5 = c.y[i] + 31.0 / 540.0 * k1[i] + 190.0 / 297.0 * k3[i] - 145.0 / 108.0 * k4[i] +
                      351.0 / 220.0 * k5[i] + 1.0 / 20.0 * k6;
    const double ym = c.y[i] + 19.0 / 216.0 * k1[i] + 1000.0 / 2079.0 * k3[i] - 125.0 / 216.0 * k4[i] +
                      81.0 / 88.0 * k5[i] + 5.0 / 56.0 * k6;
    const double err = fabs((ym - y5) * 0.2 * gw_errweight(i));
    if (err < huge_number) tr = fmax_ref(err, tr);
    else bad = true;
    finite = finite && isfinite(y5);
    c.y5[i] = y5;
  }
  // dp_after's running maximum: huge_number once any error is not below it
  tr = warp_max_ref(tr);
  if (__any_sync(0xffffffffu, bad)) tr = huge_number;
  finite = __all_sync(0xffffffffu, finite);
  __syncwarp();
  const gw_settings& P = c.set;
  if ((tr < P.tolrk || step <= P.step_min) && !finite) {
    // an accepted state that is not finite would only be accepted again at
    // the minimum step, forever: the cell stops with an error instead
    if (lane == 0) c.err = 2;
    __syncwarp();
    return;
  }
  const double tstep = c.tstep, ostep0 = c.ostep;
  bool finished_output = false;
  double nstart = start, nstep = step, nostep = ostep0;
  if (tr < P.tolrk || step <= P.step_min) {
    // accept (a forced one at the minimum step too)
    for (int i = lane; i < GW_NSTATE; i += 32) {
      double y5 = c.y5[i];
      if (fabs(y5) < min_tolvalue) y5 = 0.0;
      c.y[i] = y5;
    }
    nstart = start + step;
    if (tr < P.tolrk) {
      if (nstart >= tstep) {
        finished_output = true;
      } else {
        double ns = fmin_ref(0.85 * step * pow(P.tolrk / tr, 0.2), 4.0 * step);
        nostep = ns;
        double tts = P.shift - fmod(nstart, P.period);
        if (tts < 0.0) tts = tts + P.period;
        if (tts < ns) ns = fmax_ref(P.step_min, tts - 0.5 * P.step_min);
        nstep = ns;
      }
    } else {
      if (nstart >= tstep) finished_output = true;
      else nstep = P.step_min;
      nostep = nstep;
    }
    if (!finished_output && !(tr < P.tolrk)) {
      // the forced-accept branch clamps like a rejection (rk_pd54m.c:329-331)
      nstep = fmin_ref(P.step_max, fmax_ref(P.step_min, nstep));
      nstep = fmin_ref(nstep, tstep - nstart);
    }
    if (lane == 0) {
      c.start = nstart;
      c.success = 1;
      c.step = nstep;
      c.ostep = nostep;
      c.oldstep = nostep;
    }
    __syncwarp();
  } else {
    // reject: roll the FRUs back and retry from stage 2 (no new flux/save)
    double ns = 0.85 * step * pow(P.tolrk / tr, 0.2);
    double tts = P.shift - fmod(start, P.period);
    if (tts < 0.0) tts = tts + P.period;
    if (tts < ns) ns = fmax_ref(P.step_min, tts - 0.5 * P.step_min);
    ns = fmin_ref(P.step_max, fmax_ref(P.step_min, ns));
    ns = fmin_ref(ns, tstep - start);
    if (lane == 0) {
      c.success = 0;
      c.pending = kFlagResume;
      c.step = ns;
      c.oldstep = ostep0;
    }
    __syncwarp();
    launch_stage2_warp(c, ns, lane);
    return;
  }
  if (!finished_output) {
    if (lane == 0) {
      launch_flux(c, false);
      c.phase = kPhFlux;
    }
    __syncwarp();
    return;
  }
  // an output step is complete (gw_run): record it and start the next one
  const int k = c.step_index;
  if (c.tr_states)
    for (int i = lane; i < GW_NSTATE; i += 32) c.tr_states[(size_t)k * GW_NSTATE + i] = c.y[i];
  if (c.tr_cur)
    for (int i = lane; i < GW_NCUR; i += 32) c.tr_cur[(size_t)k * GW_NCUR + i] = c.cur[i];
  __syncwarp();
  if (lane == 0) {
    c.step_index = k + 1;
    c.steps_left--;
    c.tnow = c.tnow + P.time_step;
    if (c.steps_left <= 0) c.final_avg = 1;
    else begin_output_step(c);
    launch_flux(c, c.tr_other != nullptr || c.final_avg);
    c.phase = kPhFlux;
    if (c.final_avg && !c.tr_other) c.done = 1;
  }
  __syncwarp();
}

}  // namespace gw
