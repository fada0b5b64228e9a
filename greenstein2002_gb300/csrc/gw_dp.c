/*
 * Host side of the global step: adaptive Dormand-Prince 5(4) over the 37
 * global states, with every FRU stage on the GPU through the native C-ABI.
 * Also the whole-cell run loop (caf.c main loop) and rest initial conditions.
 *
 * Reference: rk_pd54m.c:29-345 (integrator, including its step-size rules:
 * accepted steps are not re-clamped to [step_min, step_max] within one call,
 * only rejected ones are), fcn.c:1077-1092 (lastcall), caf.c:150-255 (main
 * loop and output cadence), initialize_state.c:164-246 (rest state).
 *
 * Compiled with -ffp-contract=off: every expression keeps the reference's
 * association so that, given the same FRU fluxes, the global trajectory is
 * the reference's to the last bit wherever libm agrees.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gw_cell_model.h"
#include "gw_fru.h"

#define NS GW_NSTATE
#define GW_MIN(a, b) ((a) < (b) ? (a) : (b))
#define GW_MAX(a, b) ((a) < (b) ? (b) : (a))

void gw_settings_init(gw_settings *s) { gw_protocol_defaults(s); }

/* Error reporting of the library that links this file (gw_abi.cu, or a
 * test stand-in). */
int gw_internal_error(int code, const char *msg);

static int gw_dp_error(double t, int i)
{
    char msg[96];
    snprintf(msg, sizeof msg, "gw_rk54pd: global state %d not finite at t = %.9g ms", i, t);
    return gw_internal_error(GW_EINVAL, msg);
}

static void dep_of(const double *y, double d[3])
{
    d[0] = y[GW_V];
    d[1] = y[GW_Cai];
    d[2] = y[GW_CaNSR];
}

int gw_rk54pd(gw_ctx *ctx, const gw_settings *P, double t, double tstep, double oldstepsize, double *state,
              double *current, double *next_step)
{
    double F[NS], F1[NS], y1[NS], ym[NS], k1[NS], k2[NS], k3[NS], k4[NS], k5[NS], k6[NS];
    double dep0[3], depf[3], J[4], dummy[GW_NCUR];
    double start, st, et, step, ostep, tr, err;
    const double huge_number = 1e99, min_tolvalue = 1.e-10;
    int notdone = 1, success = 1, keepc = 1, i, rc;

    step = GW_MIN(oldstepsize, tstep - t);
    step = GW_MIN(P->step_max, step);
    ostep = step;
    start = t;
    while (notdone) {
        dep_of(state, dep0);
        if (success) {
            if ((rc = gw_flux(ctx, dep0, J, NULL))) return rc;
            gw_fcn(start, state, F1, current, keepc, J[0], J[1], J[2], J[3], P);
            keepc = 0;
            if ((rc = gw_save(ctx))) return rc;
        }
        /* stage 2: node 1/5 */
        for (i = 0; i < NS; i++) {
            k1[i] = step * F1[i];
            y1[i] = state[i] + k1[i] / 5.0;
        }
        dep_of(y1, depf);
        et = start + step / 5.0;
        if ((rc = gw_stage(ctx, start, et, dep0, depf, J, NULL))) return rc;
        dep_of(state, dep0);
        gw_fcn(start + step / 5.0, y1, F, dummy, 0, J[0], J[1], J[2], J[3], P);
        /* stage 3: node 3/10 */
        for (i = 0; i < NS; i++) {
            k2[i] = step * F[i];
            y1[i] = state[i] + (3.0 / 40.0 * k1[i] + 9.0 / 40.0 * k2[i]);
        }
        dep_of(y1, depf);
        st = start + step / 5.0;
        et = start + step * 3.0 / 10.0;
        if ((rc = gw_stage(ctx, st, et, dep0, depf, J, NULL))) return rc;
        dep_of(state, dep0);
        gw_fcn(start + step * 3.0 / 10.0, y1, F, dummy, 0, J[0], J[1], J[2], J[3], P);
        /* stage 4: node 3/5 */
        for (i = 0; i < NS; i++) {
            k3[i] = step * F[i];
            y1[i] = state[i] + (3.0 / 10.0 * k1[i] - 9.0 / 10.0 * k2[i] + 6.0 / 5.0 * k3[i]);
        }
        dep_of(y1, depf);
        st = start + step * 3.0 / 10.0;
        et = start + step * 3.0 / 5.0;
        if ((rc = gw_stage(ctx, st, et, dep0, depf, J, NULL))) return rc;
        dep_of(state, dep0);
        gw_fcn(start + step * 3.0 / 5.0, y1, F, dummy, 0, J[0], J[1], J[2], J[3], P);
        /* stage 5: node 2/3 */
        for (i = 0; i < NS; i++) {
            k4[i] = F[i] * step;
            y1[i] = state[i] + 226.0 / 729.0 * k1[i] - 25.0 / 27.0 * k2[i] + 880.0 / 729.0 * k3[i] +
                    55.0 / 729.0 * k4[i];
        }
        dep_of(y1, depf);
        st = start + step * 3.0 / 5.0;
        et = start + step * 2.0 / 3.0;
        if ((rc = gw_stage(ctx, st, et, dep0, depf, J, NULL))) return rc;
        dep_of(state, dep0);
        gw_fcn(start + step * 2.0 / 3.0, y1, F, dummy, 0, J[0], J[1], J[2], J[3], P);
        /* stage 6: node 1 */
        for (i = 0; i < NS; i++) {
            k5[i] = step * F[i];
            y1[i] = state[i] - 181.0 / 270.0 * k1[i] + 5.0 / 2.0 * k2[i] - 266.0 / 297.0 * k3[i] -
                    91.0 / 27.0 * k4[i] + 189.0 / 55.0 * k5[i];
        }
        dep_of(y1, depf);
        st = start + step * 2.0 / 3.0;
        et = start + step;
        if ((rc = gw_stage(ctx, st, et, dep0, depf, J, NULL))) return rc;
        gw_fcn(start + step, y1, F, dummy, 0, J[0], J[1], J[2], J[3], P);
        for (i = 0; i < NS; i++) k6[i] = step * F[i];
        /* 5th / 4th order solutions and the weighted max error, rk_pd54m.c:225-238 */
        tr = 0.0;
        for (i = 0; i < NS; i++) {
            y1[i] = state[i] + 31.0 / 540.0 * k1[i] + 190.0 / 297.0 * k3[i] - 145.0 / 108.0 * k4[i] +
                    351.0 / 220.0 * k5[i] + 1.0 / 20.0 * k6[i];
            ym[i] = state[i] + 19.0 / 216.0 * k1[i] + 1000.0 / 2079.0 * k3[i] - 125.0 / 216.0 * k4[i] +
                    81.0 / 88.0 * k5[i] + 5.0 / 56.0 * k6[i];
            err = fabs((ym[i] - y1[i]) * 0.2 * gw_errweight(i));
            if (err < huge_number) tr = GW_MAX(err, tr);
            else tr = huge_number;
        }
        if (tr < P->tolrk || step <= P->step_min) {
            /* a state that is not finite would only be accepted again at the
             * minimum step, forever (the reference crawls on): stop instead */
            for (i = 0; i < NS; i++)
                if (!isfinite(y1[i])) return gw_dp_error(start, i);
        }
        if (tr < P->tolrk) {
            /* accept, rk_pd54m.c:241-286 */
            for (i = 0; i < NS; i++) {
                if (fabs(y1[i]) < min_tolvalue) y1[i] = 0.0;
                state[i] = y1[i];
            }
            start = start + step;
            success = 1;
            if (start >= tstep) {
                notdone = 0;
            } else {
                double tts;
                step = GW_MIN(0.85 * step * pow(P->tolrk / tr, 0.2), 4.0 * step);
                notdone = 1;
                ostep = step;
                tts = P->shift - fmod(start, P->period);
                if (tts < 0.0) tts = tts + P->period;
                if (tts < step) step = GW_MAX(P->step_min, tts - 0.5 * P->step_min);
            }
        } else {
            if (step <= P->step_min) {
                /* forced accept at the minimum step, rk_pd54m.c:291-309 */
                for (i = 0; i < NS; i++) {
                    if (fabs(y1[i]) < min_tolvalue) y1[i] = 0.0;
                    state[i] = y1[i];
                }
                start = start + step;
                success = 1;
                if (start >= tstep) {
                    notdone = 0;
                } else {
                    step = P->step_min;
                    notdone = 1;
                }
                ostep = step;
            } else {
                /* reject and roll the FRUs back, rk_pd54m.c:315-328 */
                double tts;
                step = 0.85 * step * pow(P->tolrk / tr, 0.2);
                tts = P->shift - fmod(start, P->period);
                if (tts < 0.0) tts = tts + P->period;
                if (tts < step) step = GW_MAX(P->step_min, tts - 0.5 * P->step_min);
                success = 0;
                notdone = 1;
                if ((rc = gw_resume(ctx))) return rc;
            }
            step = GW_MIN(P->step_max, GW_MAX(P->step_min, step));
            step = GW_MIN(step, tstep - start);
        }
        oldstepsize = ostep;
    }
    if (next_step) *next_step = oldstepsize;
    return GW_OK;
}

int gw_lastcall(gw_ctx *ctx, const gw_settings *P, double time, double *state, double *current)
{
    double F[NS], dep[3], J[4];
    int rc;
    dep_of(state, dep);
    if ((rc = gw_flux(ctx, dep, J, NULL))) return rc;
    gw_fcn(time, state, F, current, 1, J[0], J[1], J[2], J[3], P);
    return GW_OK;
}

int gw_run(gw_ctx *ctx, const gw_settings *P, double *t, double *state, double *oldstep, int n_steps,
           double *states, double *other, double *currents)
{
    double cur[GW_NCUR], num[11];
    int k, rc;
    for (k = 0; k < n_steps; k++) {
        const double tnow = *t, tstep = tnow + P->time_step;
        if ((rc = gw_rk54pd(ctx, P, tnow, tstep, *oldstep, state, cur, oldstep))) return rc;
        if (other) {
            if ((rc = gw_avg_sums(ctx, num))) return rc;
            gw_otherstates(num, gw_nfru(ctx), 12500.0 / (double)gw_nfru(ctx), state, other + (size_t)k * GW_NOTHER);
        }
        if (currents) memcpy(currents + (size_t)k * GW_NCUR, cur, sizeof cur);
        if (states) memcpy(states + (size_t)k * NS, state, NS * sizeof(double));
        *t = tnow + P->time_step;
    }
    return GW_OK;
}

int gw_init_rest(gw_ctx *ctx, const gw_settings *P, int scheme, uint32_t base, double *state)
{
    const int n = gw_nfru(ctx);
    const double scale = 12500.0 / (double)n;
    double *frus;
    int *ltype, *ryr, *ito2, *mti, f, c, k, rc;
    uint32_t *mt;
    double a1 = 0.0, a2 = 0.0;
    frus = (double *)malloc(sizeof(double) * 5 * (size_t)n);
    ltype = (int *)malloc(sizeof(int) * 8 * (size_t)n);
    ryr = (int *)malloc(sizeof(int) * 20 * (size_t)n);
    ito2 = (int *)malloc(sizeof(int) * 4 * (size_t)n);
    mti = (int *)malloc(sizeof(int) * (size_t)n);
    mt = (uint32_t *)calloc((size_t)624 * n, sizeof(uint32_t));
    if (!frus || !ltype || !ryr || !ito2 || !mti || !mt) {
        free(frus); free(ltype); free(ryr); free(ito2); free(mti); free(mt);
        return GW_ENOMEM;
    }
    /* initialize_state.c:205-219 */
    for (f = 0; f < n; f++) {
        for (c = 0; c < 4; c++) {
            ltype[8 * f + 2 * c] = 1;
            ltype[8 * f + 2 * c + 1] = 2;
            for (k = 0; k < 5; k++) ryr[20 * f + 5 * c + k] = 1;
            ito2[4 * f + c] = 2;
        }
        frus[5 * f] = 0.7;
        for (c = 1; c < 5; c++) frus[5 * f + c] = 0.12e-3;
        mti[f] = 624;
    }
    rc = gw_upload(ctx, frus, ltype, ryr, ito2, mti, mt);
    if (!rc) rc = gw_seed(ctx, scheme, base);
    if (!rc) {
        gw_rest_state(state);
        if (P->vclamp_flag) state[GW_V] = P->vclamp_hold;
        if (P->iv_flag) state[GW_V] = P->iv_clamp_hold;
        /* total cell Ca, initialize_state.c:233-246 */
        for (f = 0; f < n; f++) {
            a1 = a1 + frus[5 * f] * (1.0 + GWC_CSQNtot / (GWC_KmCSQN + frus[5 * f]));
            for (c = 0; c < 4; c++)
                a2 = a2 + frus[5 * f + c + 1] *
                              (1.0 + GWC_BSRtot / (GWC_KBSR + frus[5 * f + c + 1]) +
                               GWC_BSLtot / (GWC_KBSL + frus[5 * f + c + 1]));
        }
        state[GW_CaTOT] = gw_catot(a1, a2, scale, state);
        if (P->vclamp_flag) state[GW_V] = P->vclamp_hold;
    }
    free(frus); free(ltype); free(ryr); free(ito2); free(mti); free(mt);
    return rc;
}
