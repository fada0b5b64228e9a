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

#ifdef __cplusplus
}
#endif

#endif /* GW_DIAG_H */
