/*
 * gw_diag.h -- diagnostic probes of libgw_fru.so (not part of the public
 * C-ABI in include/gw_fru.h; no reference counterpart).  They measure the
 * device arithmetic the FRU path is built on, for tests and for the design
 * notes, and are exported by the library under these names.
 */
#ifndef GW_DIAG_H
#define GW_DIAG_H

#ifdef __cplusplus
extern "C" {
#endif

/* Microseconds per evaluation of the global right-hand side (fcn.c) on one
 * GPU thread and on the host: what a device-resident integrator pays per
 * stage on GB300's FP64 rate. */
int gw_probe_fcn(double *device_us, double *host_us);
/* The same cost with the whole warp: fcn's exponentials, logs and powers
 * one per lane, then the arithmetic that combines them. */
int gw_probe_fcn_warp(double *us);
/* fcn of n states (states[n][37]) at `time` (clamp != 0: under a -100 / 0
 * mV voltage clamp) on one GPU thread and on a warp: derivatives
 * Fs/Fw[n][37] and currents Cs/Cw[n][24] of both. */
int gw_probe_fcn_compare(const double *states, int n, double time, int clamp, double *Fs, double *Fw, double *Cs,
                         double *Cw);
/* exp() of n arguments as the device evaluates it and with the host libm:
 * exp is the FRU path's only transcendental, and the two may round
 * differently in the last place. */
int gw_probe_exp(const double *x, double *device_y, double *host_y, int n);
/* FP64 issue cost on one SM, cycles per operation of warp 0 (clock64 over
 * chains of 4096 operations), in this order:
 *   [0..3]   dependent DFMA, 1 warp, 32 / 16 / 4 / 1 active lanes
 *   [4..7]   dependent DFMA, 32 lanes, 1 / 2 / 4 / 8 warps per SM
 *   [8..10]  8 independent DFMA chains per thread, 1 / 4 / 16 warps per SM
 *            (cycles per DFMA per warp)
 *   [11..12] dependent 1/x + c (DDIV + DADD), 32 / 1 active lanes
 *   [13..14] dependent exp(), 32 / 1 active lanes
 *   [15]     dependent FFMA (FP32), 1 warp */
#define GW_PROBE_ISSUE_N 16
int gw_probe_fp64_issue(double cycles[GW_PROBE_ISSUE_N]);
/* The FRU kernels' FP64 division on the integer pipe (gw_intdiv.h) against
 * the hardware division, on n operand pairs the device draws from `seed`
 * (half arbitrary bit patterns, half normal operands of magnitude
 * 1e-8 .. 1e4); *mismatches counts quotients whose bits differ. */
int gw_probe_div(unsigned long long seed, long long n, unsigned long long *mismatches);
/* The persistent kernel's wait limit, exercised without a fault: one cell
 * (its current FRU state, globals at rest) runs its first operation, after
 * which a flag that nothing sets keeps its next operation from being posted;
 * every warp then waits until nothing has progressed for wait_s seconds
 * (0 < wait_s <= 10), sets the error status and returns.  Returns GW_OK
 * when the launch ended that way, with *status = 3 (the watchdog status). */
typedef struct gw_ctx gw_ctx;
typedef struct gw_settings gw_settings;
int gw_probe_persist_watchdog(gw_ctx *cell, const gw_settings *set, double wait_s, int *status);

#ifdef __cplusplus
}
#endif

#endif /* GW_DIAG_H */
