/*
 * Harness shim linked around the reference build (test infrastructure only).
 *
 * This file is compiled inside each oracle/_ref/<config>/ tree next to the
 * reference's own sources and its (patched) parameters.h. It never ships with
 * the product. Two roles:
 *
 *  GW_SHIM_EXE  -- linked into the serial reference executable with
 *                  -Wl,--wrap=<fn> for the FRU-layer entry points that
 *                  caf.c / rk_pd54m.c / fcn.c call (mpi_master.c:41,122,199,
 *                  369,477,493,643; initialize_ran.c:23; fcn.c:29 when it
 *                  stores currents).  The wrappers log
 *                  every call (inputs and outputs) to the binary file named
 *                  by $GW_REF_LOG and dump the initial / final FRU working set
 *                  (the *_local globals of mpi_slave.c:31-45) to
 *                  $GW_REF_DUMP_INIT / $GW_REF_DUMP_FINAL.  With $GW_SEED_BASE
 *                  set, FRU j is seeded with sgrnd_local(base + j) instead of
 *                  the reference formula of initialize_ran.c:30-34.
 *
 *  GW_SHIM_LIB  -- linked into libref.so together with the reference's
 *                  per-FRU routines, so tests can call simfru_local, fcn,
 *                  the MT19937 routines and the flux/average sums on arrays
 *                  they own (ctypes).  It defines the globals caf.c:27-38
 *                  would otherwise provide.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "parameters.h"

/* ------------------------------------------------------------------------ */
/* dump format: int32 n, then f64 FRU[n][5], i32 LType[n][4][2],            */
/* i32 RyR[n][4][5], i32 Ito2[n][4], i32 mti[n], u32 mt[n][624]             */
/* ------------------------------------------------------------------------ */
static void dump_local_set(const char *path)
{
    FILE *f;
    int n = NFRU_local, i, k;
    if (!path || !*path) return;
    f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "shim: cannot open %s\n", path); abort(); }
    fwrite(&n, sizeof(int), 1, f);
    for (i = 0; i < n; i++) fwrite(&FRU_states_local[i][0], sizeof(double), Nstates_FRU, f);
    for (i = 0; i < n; i++) fwrite(&LType_state_local[i][0][0], sizeof(int), Nclefts_FRU * Nindepstates_LType, f);
    for (i = 0; i < n; i++) fwrite(&RyR_state_local[i][0][0], sizeof(int), Nclefts_FRU * NRyRs_per_cleft, f);
    for (i = 0; i < n; i++) fwrite(&Ito2_state_local[i][0], sizeof(int), Nclefts_FRU, f);
    fwrite(&mti_local[0], sizeof(int), n, f);
    for (i = 0; i < n; i++)
        for (k = 0; k < mtN; k++) {
            uint32_t w = (uint32_t)mt_local[i][k];
            fwrite(&w, sizeof(uint32_t), 1, f);
        }
    fclose(f);
}

#ifdef GW_SHIM_EXE
static FILE *logf_;
static void log_open(void)
{
    const char *p;
    if (logf_) return;
    p = getenv("GW_REF_LOG");
    if (p && *p) {
        logf_ = fopen(p, "wb");
        if (!logf_) { fprintf(stderr, "shim: cannot open %s\n", p); abort(); }
    }
}
static void log_rec(char tag, const double *v, int n)
{
    log_open();
    if (!logf_) return;
    fputc(tag, logf_);
    if (n) fwrite(v, sizeof(double), (size_t)n, logf_);
}

void __real_initialize_ran(unsigned long mt[NFRU_sim_max][mtN + 1], int mti[NFRU_sim_max]);
void __wrap_initialize_ran(unsigned long mt[NFRU_sim_max][mtN + 1], int mti[NFRU_sim_max])
{
    const char *b = getenv("GW_SEED_BASE");
    if (b && *b) {
        unsigned long base = strtoul(b, NULL, 10);
        int j;
        for (j = 0; j < NFRU_sim; j++) sgrnd_local((base + (unsigned long)j) & 0xffffffffUL, &mti[j], &mt[j][0]);
    } else {
        __real_initialize_ran(mt, mti);
    }
}

void __real_initialize_mpi_state(double a[NFRU_sim_max][Nstates_FRU], int b[NFRU_sim_max][Nclefts_FRU][Nindepstates_LType],
                                 int c[NFRU_sim_max][Nclefts_FRU][NRyRs_per_cleft], int d[NFRU_sim_max][Nclefts_FRU],
                                 int e[NFRU_sim_max], unsigned long g[NFRU_sim_max][mtN + 1]);
void __wrap_initialize_mpi_state(double a[NFRU_sim_max][Nstates_FRU], int b[NFRU_sim_max][Nclefts_FRU][Nindepstates_LType],
                                 int c[NFRU_sim_max][Nclefts_FRU][NRyRs_per_cleft], int d[NFRU_sim_max][Nclefts_FRU],
                                 int e[NFRU_sim_max], unsigned long g[NFRU_sim_max][mtN + 1])
{
    __real_initialize_mpi_state(a, b, c, d, e, g);
    dump_local_set(getenv("GW_REF_DUMP_INIT"));
    log_rec('I', NULL, 0);
}

void __real_distrib_simFRU(double, double, double[Nstates_FRUdep], double[Nstates_FRUdep], double *, double *, double *, double *);
void __wrap_distrib_simFRU(double st, double et, double d0[Nstates_FRUdep], double df[Nstates_FRUdep],
                           double *Jxfer, double *Jtr, double *ICa, double *Ito2)
{
    double rec[12];
    rec[0] = st; rec[1] = et;
    memcpy(&rec[2], d0, 3 * sizeof(double));
    memcpy(&rec[5], df, 3 * sizeof(double));
    __real_distrib_simFRU(st, et, d0, df, Jxfer, Jtr, ICa, Ito2);
    rec[8] = *Jxfer; rec[9] = *Jtr; rec[10] = *ICa; rec[11] = *Ito2;
    log_rec('S', rec, 12);
}

void __real_send_calc_fru_flux(double[Nstates_FRUdep], double *, double *, double *, double *);
void __wrap_send_calc_fru_flux(double d[Nstates_FRUdep], double *Jxfer, double *Jtr, double *ICa, double *Ito2)
{
    double rec[7];
    memcpy(rec, d, 3 * sizeof(double));
    __real_send_calc_fru_flux(d, Jxfer, Jtr, ICa, Ito2);
    rec[3] = *Jxfer; rec[4] = *Jtr; rec[5] = *ICa; rec[6] = *Ito2;
    log_rec('F', rec, 7);
}

void __real_send_calc_fru_avg(double[N], double[Nother]);
void __wrap_send_calc_fru_avg(double state[N], double other[Nother])
{
    double rec[N + Nother];
    __real_send_calc_fru_avg(state, other);
    memcpy(rec, state, N * sizeof(double));
    memcpy(rec + N, other, Nother * sizeof(double));
    log_rec('A', rec, N + Nother);
}

void __real_send_save_state(void);
void __wrap_send_save_state(void) { log_rec('V', NULL, 0); __real_send_save_state(); }
void __real_send_resume_state(void);
void __wrap_send_resume_state(void) { log_rec('R', NULL, 0); __real_send_resume_state(); }

void __real_fcn(const double, double[N], double[N], double[Ncur], const int, const double, const double,
                const double, const double);
void __wrap_fcn(const double t, double state[N], double F[N], double cur[Ncur], const int keepc, const double Jxfer,
                const double Jtr, const double ICa, const double Ito2)
{
    __real_fcn(t, state, F, cur, keepc, Jxfer, Jtr, ICa, Ito2);
    if (keepc) {
        double rec[1 + Ncur];
        rec[0] = t;
        memcpy(rec + 1, cur, Ncur * sizeof(double));
        log_rec('C', rec, 1 + Ncur);
    }
}

void __real_end_mpi(void);
void __wrap_end_mpi(void)
{
    dump_local_set(getenv("GW_REF_DUMP_FINAL"));
    log_rec('E', NULL, 0);
    if (logf_) { fclose(logf_); logf_ = NULL; }
    __real_end_mpi();
}
#endif /* GW_SHIM_EXE */

#ifdef GW_SHIM_LIB
/* Globals that caf.c:27-38 defines in the full program. */
double time_of_last_change, glob_time_to_stim;
int current_phase;
double surand_seed[NFRU_sim_max];
double errweight[N];
int iv_n;
double NFRU_scale;
double NFRU_sim_factor;
int NFRU_sim;
int my_rank;
int procs = 1;

/* Advance n FRUs over [t0,tf] with the reference's simfru_local.
 * Arrays are packed per FRU: ltype[n][4][2], ryr[n][4][5], ito2[n][4],
 * frus[n][5], mti[n], mt32[n][624] (MT words as uint32). */
void ref_simfru_batch(int n, double t0, double tf, const double dep0[3], const double depf[3],
                      int *ltype, int *ryr, int *ito2, double *frus, int *mti, uint32_t *mt32)
{
    static unsigned long mtw[mtN + 1];
    double d0[3], df[3];
    int i, k;
    for (i = 0; i < n; i++) {
        memcpy(d0, dep0, sizeof d0);
        memcpy(df, depf, sizeof df);
        for (k = 0; k < mtN; k++) mtw[k] = mt32[(size_t)i * mtN + k];
        simfru_local(t0, tf, d0, df,
                     (int(*)[Nindepstates_LType])(ltype + (size_t)i * 8),
                     (int(*)[NRyRs_per_cleft])(ryr + (size_t)i * 20),
                     ito2 + (size_t)i * 4, frus + (size_t)i * 5, &mti[i], mtw);
        for (k = 0; k < mtN; k++) mt32[(size_t)i * mtN + k] = (uint32_t)mtw[k];
    }
}

/* Reference rate tables for one FRU (fru_rates_local.c:30); may draw. */
double ref_fru_rates(int *ltype, int *ryr, int *ito2, const double dep[3], const double frus[5],
                     double *lrates, int *lindex, int *llen, double *vdep, double *rrates, int *rindex,
                     int *rlen, double *ito2rate, int *mti, uint32_t *mt32)
{
    static unsigned long mtw[mtN + 1];
    double r;
    int k;
    for (k = 0; k < mtN; k++) mtw[k] = mt32[k];
    r = fru_rates_local((int(*)[Nindepstates_LType])ltype, (int(*)[NRyRs_per_cleft])ryr, ito2, dep, frus,
                        (double(*)[4])lrates, (int(*)[4])lindex, llen, vdep,
                        (double(*)[NRyRs_per_cleft][4])rrates, (int(*)[NRyRs_per_cleft][4])rindex,
                        (int(*)[NRyRs_per_cleft])rlen, ito2rate, mti, mtw);
    for (k = 0; k < mtN; k++) mt32[k] = (uint32_t)mtw[k];
    return r;
}

void ref_fcn_fru(double t, const double frus[5], const double dep[3], const double lopen[4],
                 const int nryr[4], double out[5])
{
    fcn_fru(t, frus, dep, lopen, nryr, out);
}

void ref_sgrnd(unsigned long seed, int *mti, uint32_t *mt32)
{
    unsigned long mtw[mtN + 1];
    int k;
    sgrnd_local(seed, mti, mtw);
    for (k = 0; k < mtN; k++) mt32[k] = (uint32_t)mtw[k];
}

/* n uniforms through MersenneTwister_fast (mt19937_local.c:97). */
void ref_mt_fast(int n, int *mti, uint32_t *mt32, double *out)
{
    unsigned long mtw[mtN + 1];
    int k;
    for (k = 0; k < mtN; k++) mtw[k] = mt32[k];
    MersenneTwister_fast(mti, mtw, n, out);
    for (k = 0; k < mtN; k++) mt32[k] = (uint32_t)mtw[k];
}

double ref_mt_one(int *mti, uint32_t *mt32)
{
    unsigned long mtw[mtN + 1];
    double r;
    int k;
    for (k = 0; k < mtN; k++) mtw[k] = mt32[k];
    r = MersenneTwisterOne_local(mti, mtw);
    for (k = 0; k < mtN; k++) mt32[k] = (uint32_t)mtw[k];
    return r;
}

/* Seeds of initialize_ran.c:23 for n FRUs: mti[n], mt32[n][624]. */
void ref_initialize_ran(int n, int *mti, uint32_t *mt32)
{
    static unsigned long mtw[NFRU_sim_max][mtN + 1];
    static int mtiw[NFRU_sim_max];
    int i, k;
    NFRU_sim = n;
    initialize_ran(mtw, mtiw);
    for (i = 0; i < n; i++) {
        mti[i] = mtiw[i];
        for (k = 0; k < mtN; k++) mt32[(size_t)i * mtN + k] = (uint32_t)mtw[i][k];
    }
}

void ref_fcn(double t, double *state, double *F, double *current, int keepc,
             double Jxfer, double Jtr, double ICa, double Ito2)
{
    fcn(t, state, F, current, keepc, Jxfer, Jtr, ICa, Ito2);
}

/* Flux numerators of calc_fru_flux_local.c:28 over packed arrays. */
void ref_flux_sums(int n, int *ltype, int *ito2, double *frus, double num[5])
{
    calc_fru_flux_local(n, (int(*)[Nclefts_FRU][Nindepstates_LType])ltype, (int(*)[Nclefts_FRU])ito2,
                        (double(*)[Nstates_FRU])frus, num);
}

/* Output sums of calc_fru_avg_local.c:27 over packed arrays. */
void ref_avg_sums(int n, int *ltype, int *ryr, int *ito2, double *frus, double num[11])
{
    calc_fru_avg_local(num, n, (double(*)[Nstates_FRU])frus, (int(*)[Nclefts_FRU][Nindepstates_LType])ltype,
                       (int(*)[Nclefts_FRU][NRyRs_per_cleft])ryr, (int(*)[Nclefts_FRU])ito2);
}
#endif /* GW_SHIM_LIB */
