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

}  // namespace gw
