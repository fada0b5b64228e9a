/*
 * gw_fru.h -- C-ABI of the GB300 FRU hot path (libgw_fru.so).
 *
 * Two layers, both plain C (no CUDA or torch types in any signature):
 *
 *  1. The drop-in layer: the FRU-distribution entry points of the reference's
 *     MPI layer with their exact names and signatures (declared in the
 *     reference's parameters.h:255-271).  A program built from the reference's
 *     caf.c / rk_pd54m.c / fcn.c links against this library instead of
 *     mpi_master.c + mpi_slave.c and runs its FRUs on the GPU.  Each call
 *     aborts with a message on a CUDA error, as the reference aborts on I/O
 *     errors.  NFRU_sim and NFRU_scale are read from the program's globals
 *     (caf.c:34-36) when it defines them, else from gw_dropin_configure().
 *
 *  2. The native layer (gw_*): explicit context, runtime settings, int status
 *     codes, multi-cell capable.  The drop-in layer is built on it.
 *
 * Array layouts are the reference's: per FRU ltype[4][2], ryr[4][5], ito2[4],
 * frus[5] (CaJSR, CaSS1..4), mti, and 624 MT19937 state words.
 */
#ifndef GW_FRU_H
#define GW_FRU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------- */
/* Status codes                                                               */
/* ------------------------------------------------------------------------- */
#define GW_OK 0
#define GW_EINVAL 1     /* bad argument (size, pointer, state value) */
#define GW_ECUDA 2      /* CUDA runtime error (message via gw_last_error) */
#define GW_ENOMEM 3     /* device or host allocation failed */
#define GW_ENODEV 4     /* no usable GPU */

const char *gw_last_error(void);

/* ------------------------------------------------------------------------- */
/* Native layer                                                               */
/* ------------------------------------------------------------------------- */
typedef struct gw_ctx gw_ctx;

/* Cell of nfru FRUs on the current CUDA device (replaces the per-rank FRU
 * blocks of initialize_mpi_state, mpi_master.c:199-361). */
int gw_create(gw_ctx **ctx, int nfru);
int gw_destroy(gw_ctx *ctx);
int gw_nfru(const gw_ctx *ctx);

/* Flux scale factor 12500/NFRU (parameters.h:43-46) and the LCC
 * permeability scale (1.0 = reference PCa, parameters_fcn_fru.c:48). */
int gw_set_scale(gw_ctx *ctx, double nfru_scale);

/* FRU state upload / download (host arrays in the reference layout; mt as
 * uint32 words [n][624]).  Replace the scatter of initialize_mpi_state
 * (mpi_master.c:199) and the gather of parallel_get_FRUs (mpi_master.c:509). */
int gw_upload(gw_ctx *ctx, const double *frus, const int *ltype, const int *ryr, const int *ito2, const int *mti,
              const uint32_t *mt);
int gw_download(gw_ctx *ctx, double *frus, int *ltype, int *ryr, int *ito2, int *mti, uint32_t *mt);
/* The same for FRUs first .. first+count-1 only (arrays indexed from 0):
 * what write_fru_props (write_fru_props.c:28-128) reads at every output
 * step, without the whole-cell gather of parallel_get_FRUs. */
int gw_download_range(gw_ctx *ctx, int first, int count, double *frus, int *ltype, int *ryr, int *ito2);

/* Seed every FRU's MT19937 on the device: scheme 0 = seed base+j,
 * scheme 1 = the formula of initialize_ran.c:30-34. */
int gw_seed(gw_ctx *ctx, int scheme, uint32_t base);

/* One Dormand-Prince stage: advance all FRUs over [t0, tf] with V/Cai/CaNSR
 * interpolated from dep0 to depf; out = Jxfer, Jtr, ICa, Ito2 at depf.
 * num (optional, may be NULL) receives the 5 flux numerators.
 * Replaces distrib_simFRU (mpi_master.c:369-469). */
int gw_stage(gw_ctx *ctx, double t0, double tf, const double dep0[3], const double depf[3], double out[4],
             double num[5]);
/* Fluxes of the current FRU state at dep (send_calc_fru_flux, mpi_master.c:41). */
int gw_flux(gw_ctx *ctx, const double dep[3], double out[4], double num[5]);
/* The 11 output sums of calc_fru_avg_local.c:27 (send_calc_fru_avg). */
int gw_avg_sums(gw_ctx *ctx, double num[11]);
/* Snapshot / rollback of FRU + RNG state (send_save_state :477,
 * send_resume_state :493).  Applied lazily by the next device operation. */
int gw_save(gw_ctx *ctx);
int gw_resume(gw_ctx *ctx);

/* Lanes per FRU of the FP64 stage kernel: 4 (default) = one lane per cleft,
 * 8 FRUs per warp, shortest FP64 chain per FRU; 1 = one thread per FRU, 32
 * FRUs per warp.  Results are identical; the choice only changes speed. */
int gw_set_fru_lanes(gw_ctx *ctx, int lanes);
/* Warps per block of the 4-lane stage kernels: 1 (default), 2, 4 or 8.  A
 * launch-shape choice only; every value gives the same results. */
int gw_set_stage_warps(gw_ctx *ctx, int warps);
/* Packed stage launches (0 = off, the default): `warps` warps whose 4-lane
 * groups take the cell's FRUs from a queue -- the heaviest of the previous
 * launch first -- until none are left, instead of 8 fixed FRUs per warp
 * (so FRUs per warp = 8 x FRUs / (8 x warps) on average).  A launch-shape
 * choice only: every FRU ends in the same state and the flux sums keep
 * their order. */
int gw_set_stage_packing(gw_ctx *ctx, int warps);

/* Arithmetic of the FRU path: 0 (default) = FP64, the plain method;
 * 1 = mixed precision: transition rates and the FRU-local Ca ODE in FP32,
 * FP64 kept for the FRU Ca state, the FRU clock and the flux sums.  Both use
 * the same channel algorithm and the same MT19937 draws. */
int gw_set_precision(gw_ctx *ctx, int precision);
/* Per-cell scale of the LCC permeability PCa (g_CaL; 1.0 = the reference,
 * parameters_fcn_fru.c:48), applied to the LCC flux of every cleft and to ICa. */
int gw_set_pca_scale(gw_ctx *ctx, double scale);

/* Order of the cross-FRU sums (flux numerators, output sums).
 * GW_SUM_TREE (default): one fixed parallel tree, the same bits for every
 * launch shape.  GW_SUM_REFERENCE: the serial reference's order, one FRU and
 * one cleft after another (calc_fru_flux_local.c:44-70,
 * calc_fru_avg_local.c:50-91), computed by one GPU thread after each stage --
 * a parity mode for small cells, so that whole-cell trajectories can be
 * compared with the reference program bit for bit.  Single cells and
 * per-stream runs only (a lockstep batch or the device-resident integrator
 * returns GW_EINVAL for such a cell). */
#define GW_SUM_TREE 0
#define GW_SUM_REFERENCE 1
int gw_set_sum_order(gw_ctx *ctx, int order);

/* FRU-substeps executed since creation (workload counter). */
int gw_substeps(gw_ctx *ctx, unsigned long long *count);
/* Wait for all work of the context. */
int gw_sync(gw_ctx *ctx);

/* Measurement helpers on the context's stream (no reference counterpart):
 * events in slots 0..7; per-launch device time of the FRU stage kernel while
 * profiling is enabled; kernel-launch counter; an L2 flush (writes 512 MB);
 * a measured FP64 FMA peak of the device in TFLOP/s. */
int gw_event_record(gw_ctx *ctx, int slot);
int gw_event_elapsed(gw_ctx *ctx, int slot_a, int slot_b, float *ms);
int gw_profile(gw_ctx *ctx, int enable);
/* Device time of work several cells run concurrently on their own streams
 * (no reference counterpart): phase 0 before the work, phase 1 after it
 * returns the elapsed ms in *ms.  Not thread-safe; one group at a time. */
int gw_group_timer(int n, gw_ctx **cells, int phase, float *ms);
/* Stage trace (diagnostics of the 4-lane kernels; no reference
 * counterpart): when enabled, every stage launch records each FRU's substep
 * count and each 8-FRU warp's begin and end global time in ns;
 * gw_stage_trace_read returns the last launch's: substeps[nfru],
 * warp_ns[ceil(nfru/8)][2] (either may be NULL).  Enable before the cell
 * joins a batch. */
int gw_stage_trace(gw_ctx *ctx, int enable);
int gw_stage_trace_read(gw_ctx *ctx, uint32_t *substeps, unsigned long long *warp_ns);
int gw_profile_read(gw_ctx *ctx, double *stage_kernel_ms, unsigned long long *stage_launches);
int gw_launches(gw_ctx *ctx, unsigned long long *count);
int gw_l2_flush(gw_ctx *ctx);
int gw_probe_fp64_peak(double *tflops);

/* Allocation-free FRU stage (no counterpart in the reference).  For callers
 * that cannot allocate device memory while they run -- cudaMalloc
 * synchronises the device, is not allowed during stream capture, and is off
 * limits to hosts that own all device memory -- this advances FRU arrays the
 * caller owns on the device over [t0, tf] with the plain FP64 method (the
 * one-thread-per-FRU kernel, the reference PCa, no packed launches: the
 * results of gw_stage on a context with default settings) and writes
 * out[0..4] = flux sums, out[5..8] = Jxfer, Jtr, ICa, Ito2, out[9] = error
 * flag (a device or host-mapped array of 10 doubles): 1 when the substep
 * limit was reached, 2 when an FRU's mti was outside 0..624 or a channel
 * state outside its range (LCC 1..12, VDI 1..2, RyR 1..8, ClCh 1..2); such an
 * FRU is left unchanged.  Arrays use the device layout of gw_stage:
 * frus[5][stride] f64, chan[4][stride] packed channel words (LCC, VDI,
 * RyR0..4, ClCh nibbles), mti[stride], mt[nfru][640] words.
 * Its reduction scratch is a fixed array inside the library (about 80 KB per
 * GPU, held until the process exits), which limits nfru to 65,536; larger
 * cells get GW_EINVAL.  No save/resume snapshot is taken on this path.  The
 * first call on a device resolves the scratch address, so make it before any
 * stream capture.  All calls share the scratch: calls that overlap on the GPU
 * (different streams, or different cells at once) race and must be
 * serialised by the caller.  Asynchronous on `stream` (a cudaStream_t). */
int gw_stage_noalloc(int nfru, int stride, double *frus, uint32_t *chan, int *mti, uint32_t *mt, double t0, double tf,
                     const double dep0[3], const double depf[3], double nfru_scale, double *out, void *stream);

/* Run settings of parameters.h:92-156 as a runtime struct; see
 * gw_protocol_init for the defaults (the reference's parameters.h values). */
typedef struct gw_settings {
  double time_start, time_end, time_step, step_min, step_max, tolrk;
  double pulse_duration, pulse_amplitude, period, shift;
  int vclamp_flag;
  double vclamp_duration, vclamp_set, vclamp_shift, vclamp_hold, vclamp_period;
  int vppclamp_flag;
  double vppclamp_ppset, vppclamp_ppduration, vppclamp_shift, vppclamp_set, vppclamp_duration, vppclamp_hold,
      vppclamp_period;
  int iv_flag;
  double iv_clamp_duration, iv_clamp_period, iv_shift, iv_clamp_set, iv_clamp_hold, iv_clamp_step;
  int iv_n;
  int chf_flag;
  double chfsc_IK1, chfsc_Jup, chfsc_INaCa, chfsc_IKv43;
  double scale_PCa, scale_GKr;
} gw_settings;

void gw_settings_init(gw_settings *s);

/* Adaptive Dormand-Prince 5(4) over [t, tstep] with FRU stages on the GPU
 * (rk_pd54m.c:29-345).  state[37] in/out, current[24] out; returns the step
 * size to start the next call with in *next_step. */
int gw_rk54pd(gw_ctx *ctx, const gw_settings *set, double t, double tstep, double oldstepsize, double *state,
              double *current, double *next_step);
/* Final currents at `time` (fcn.c:1077). */
int gw_lastcall(gw_ctx *ctx, const gw_settings *set, double time, double *state, double *current);

/* Whole-cell run: n_steps output steps of set->time_step from *t (the main
 * loop of caf.c:150-251).  Per step k it stores states[k][37] at t+(k+1)dt,
 * other[k][12] (otherstates), currents[k][24] at t+k*dt; any of them may be
 * NULL.  *t, state, *oldstep advance in place. */
int gw_run(gw_ctx *ctx, const gw_settings *set, double *t, double *state, double *oldstep, int n_steps,
           double *states, double *other, double *currents);

/* Rest initial conditions of initialize_state.c:164-246 for the cell:
 * 37 globals (CaTOT from the FRU sums) and every FRU at rest, seeded by
 * `scheme`/`base` as in gw_seed. */
int gw_init_rest(gw_ctx *ctx, const gw_settings *set, int scheme, uint32_t base, double *state);

/* ------------------------------------------------------------------------- */
/* Batching: many cells, one stage launch per round (no reference            */
/* counterpart; the reference runs one cell per MPI job)                      */
/* ------------------------------------------------------------------------- */
typedef struct gw_batch gw_batch;
/* precision as gw_set_precision; member cells must use the same precision and
 * the default 4-lane kernel. */
int gw_batch_create(gw_batch **batch, int precision);
int gw_batch_destroy(gw_batch *batch);
/* Join / leave between rounds.  While a member, a cell's stage and flux
 * operations wait for the round in which every member has posted one; each
 * member must therefore be driven by its own host thread.  A cell's results
 * do not depend on which other cells share its rounds. */
int gw_batch_add(gw_batch *batch, gw_ctx *ctx);
int gw_batch_remove(gw_batch *batch, gw_ctx *ctx);
/* Batched-kernel device time and launches since the last call (enable != 0
 * starts measuring). */
int gw_batch_profile(gw_batch *batch, int enable, double *kernel_ms, unsigned long long *launches);
/* Run n cells for n_steps output steps each, one host thread per cell:
 * states[n][37], t[n], oldsteps[n] advance in place; state_trace
 * [n][n_steps][37] and other_trace [n][n_steps][12] (either may be NULL)
 * receive every output step's states and otherstates. */
int gw_batch_run(gw_batch *batch, int n, gw_ctx **cells, const gw_settings *sets, double *t, double *states,
                 double *oldsteps, int n_steps, double *state_trace, double *other_trace);
/* The same without shared rounds: each cell on its own stream and host
 * thread, its kernels running concurrently with the others'. */
int gw_run_concurrent(int n, gw_ctx **cells, const gw_settings *sets, double *t, double *states, double *oldsteps,
                      int n_steps, double *state_trace, double *other_trace);
/* Device-resident integrator (the level-B seam of rk54pd, rk_pd54m.c:29):
 * n cells advance n_steps output steps each with their Dormand-Prince
 * integrators on the GPU -- one CUDA graph whose WHILE loop runs rounds of
 * [every cell's FRU launch, every cell's integrator step] until all cells
 * are done; no host round trip inside a step.  Arguments as gw_batch_run,
 * plus cur_trace [n][n_steps][24] (may be NULL).  Cells must share one
 * precision and not be in a batch.  Same arithmetic as gw_run, except that
 * the global right-hand side uses CUDA's exp/pow/log (last-place
 * differences from the host C library). */
int gw_run_device(int n, gw_ctx **cells, const gw_settings *sets, double *t, double *states, double *oldsteps,
                  int n_steps, double *state_trace, double *other_trace, double *cur_trace);
/* Persistent multi-cell kernel (the level-B seam of rk54pd, rk_pd54m.c:29, and
 * the stage dispatch of distrib_simFRU, mpi_master.c:369-469, for many cells
 * at once): n cells advance n_steps output steps each inside one resident
 * launch, captured with its copy-back as one CUDA graph.  Warps take batches
 * of 8-FRU groups (1 to 4 groups, fewer for small runs; the environment
 * variable GW_PERSIST_GROUPS = 1..8 overrides) from whichever cell has an
 * open stage or flux evaluation, advance and sum them, and the warp that
 * finishes a cell's operation runs its integrator step; so no cell waits for
 * another's slowest FRU and no host thread or round trip sits inside a step.
 * Arguments as gw_run_device; cells must share one precision and not be in a
 * batch.  A cell's results are the same bits alone, in any mix, for any batch
 * size and under gw_run_device.  If no work anywhere progresses for 2 s the
 * launch ends with GW_ECUDA instead of waiting on. */
int gw_run_persistent(int n, gw_ctx **cells, const gw_settings *sets, double *t, double *states, double *oldsteps,
                      int n_steps, double *state_trace, double *other_trace, double *cur_trace);
/* Warps per block of the batch's launches (1, 2, 4 or 8; same results). */
int gw_batch_set_warps(gw_batch *batch, int warps);

/* Autotuner (no reference counterpart): runs window_ms of the cells' own
 * workload from their current state once per stage-kernel launch shape --
 * 4 lanes per FRU with 1, 2, 4 or 8 warps per block, 1 lane per FRU (FP64
 * cells with the reference PCa, not in a batch), and packed launches with
 * a half, a quarter or an eighth as many warps as the cell has 8-FRU groups
 * (not in a batch) -- then restores their state and sets the fastest shape
 * on every cell (and on the batch).  *warps receives the warps per block,
 * or -2 / -4 / -8 for the packed shapes.
 * The cells run alone (n = 1), concurrently on their own streams (batch
 * NULL) or through the batch.  t, states [n][37] and oldsteps are read, not
 * advanced.  ms (may be NULL) receives the wall time of each of the
 * GW_TUNE_CANDIDATES candidates in the order above, -1 where not run.
 * Results never depend on the shape chosen. */
#define GW_TUNE_CANDIDATES 8
int gw_autotune(int n, gw_ctx **cells, const gw_settings *sets, const double *t, const double *states,
                const double *oldsteps, double window_ms, gw_batch *batch, int *lanes, int *warps, double *ms);

/* ------------------------------------------------------------------------- */
/* Serving: requests arrive at any time and run concurrently through one     */
/* batch (continuous batching; no reference counterpart)                      */
/* ------------------------------------------------------------------------- */
typedef struct gw_request {
  int nfru;                /* FRUs of the cell */
  gw_settings set;         /* protocol (pacing or voltage clamp) and conductance scales */
  int seed_scheme;         /* as gw_seed */
  uint32_t seed;
  double pca_scale;        /* LCC permeability scale (0 or 1: the reference) */
  double duration_ms;      /* simulated time from the rest state */
  double *v_trace;         /* optional host buffer: V at every output step */
  double *final_state;     /* optional host buffer [37] */
  double t_submit, t_start, t_done; /* host clock seconds, set by the server */
  int status;              /* -1 while pending, then a GW_* status */
  char message[160];       /* the error message when status is not GW_OK */
} gw_request;
typedef struct gw_server gw_server;
/* Device bytes a cell of nfru FRUs holds (the admission unit). */
size_t gw_cell_bytes(int nfru);
/* slots worker threads; requests are admitted in arrival order.  The server
 * holds at most mem_budget_bytes of cell contexts (gw_cell_bytes each),
 * counting the running cells and the idle contexts it pools for reuse: a
 * request starts when a pooled context of its FRU count is idle, or when a
 * new one fits beside everything held, destroying idle contexts of other
 * sizes if that makes it fit.  lockstep = 1 runs the admitted cells through
 * one gw_batch; 0 gives each its own stream. */
int gw_server_create(gw_server **srv, int precision, int slots, size_t mem_budget_bytes, int lockstep);
/* Create `count` idle contexts of nfru FRUs now (within the budget), so that
 * requests of that size allocate nothing -- no device-wide synchronisation --
 * while other requests run. */
int gw_server_reserve(gw_server *srv, int nfru, int count);
/* Bytes of contexts held now and at most so far, and the context allocations
 * and frees made so far (reserve included). */
int gw_server_stats(gw_server *srv, size_t *held, size_t *peak_held, unsigned long long *allocs,
                    unsigned long long *frees);
/* Non-blocking; req must stay valid until gw_server_wait returns. */
int gw_server_submit(gw_server *srv, gw_request *req);
int gw_server_wait(gw_server *srv);
int gw_server_destroy(gw_server *srv);

/* ------------------------------------------------------------------------- */
/* Drop-in layer: reference names and signatures (parameters.h:255-271).      */
/* ------------------------------------------------------------------------- */
/* Overrides for programs that do not define the globals NFRU_sim and
 * NFRU_scale of caf.c:34-36. */
void gw_dropin_configure(int nfru, double nfru_scale);
/* The context the drop-in layer uses (created by initialize_mpi_state). */
gw_ctx *gw_dropin_context(void);

/* mpi_master.c:625 -- sets *rank = 0, *procs = 1 (one GPU, one process). */
void initialize_mpi(int *argc, char **argv, int *rank, int *procs);
/* mpi_master.c:643 -- releases the GPU context. */
void end_mpi(void);
/* mpi_master.c:199 -- uploads the first NFRU_sim FRUs.  mt rows are the
 * reference's unsigned long[625] arrays. */
void initialize_mpi_state(double FRU_states[][5], int LType_state[][4][2], int RyR_state[][4][5],
                          int Ito2_state[][4], int mti[], unsigned long mt[][625]);
/* mpi_master.c:369 */
void distrib_simFRU(double st_time, double end_time, double FRUdep_states0[3], double FRUdep_statesf[3],
                    double *Jxfer, double *Jtr, double *ICa, double *Ito2);
/* mpi_master.c:41 */
void send_calc_fru_flux(double FRUdep_states[3], double *Jxfer, double *Jtr, double *ICa, double *Ito2);
/* mpi_master.c:122 -- otherstate[12] from the FRU sums and state[37]. */
void send_calc_fru_avg(double state[37], double otherstate[12]);
/* mpi_master.c:477, :493 */
void send_save_state(void);
void send_resume_state(void);
/* mpi_master.c:509 -- downloads all FRUs into the reference's arrays. */
void parallel_get_FRUs(double FRU_states[][5], int LType_state[][4][2], int RyR_state[][4][5], int Ito2_state[][4],
                       unsigned long mt[][625], int mti[]);
/* mpi_slave.c:348 -- the worker loop; never entered with one process. */
void parallel(void);

#ifdef __cplusplus
}
#endif

#endif /* GW_FRU_H */
