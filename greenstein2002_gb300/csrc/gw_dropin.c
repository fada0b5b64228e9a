/*
 * Drop-in layer: the reference's FRU-distribution entry points (the MPI layer
 * of mpi_master.c / mpi_slave.c) with their exact names and signatures,
 * implemented on the native GPU API.  A program built from the reference's
 * caf.c, rk_pd54m.c and fcn.c links this library in place of mpi_master.c and
 * mpi_slave.c; its FRUs then live on the GPU for the whole run and only the
 * 8 stage inputs and 4 fluxes cross the host boundary per stage.
 *
 * NFRU_sim and NFRU_scale (caf.c:34-36) are read through weak references when
 * the program defines them; gw_dropin_configure() sets them otherwise.  CUDA
 * errors abort with a message, like the reference's own fatal errors.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gw_cell_model.h"
#include "gw_fru.h"

extern int NFRU_sim __attribute__((weak));
extern double NFRU_scale __attribute__((weak));

static gw_ctx *g_ctx;
static int g_nfru = -1;
static double g_scale = -1.0;

void gw_dropin_configure(int nfru, double nfru_scale)
{
    g_nfru = nfru;
    g_scale = nfru_scale;
}

gw_ctx *gw_dropin_context(void) { return g_ctx; }

static int dropin_nfru(void)
{
    if (g_nfru > 0) return g_nfru;
    if (&NFRU_sim) return NFRU_sim;
    fprintf(stderr, "gw_fru: NFRU_sim is not defined; call gw_dropin_configure()\n");
    abort();
}

static double dropin_scale(void)
{
    if (g_scale > 0.0) return g_scale;
    if (&NFRU_scale) return NFRU_scale;
    return 12500.0 / (double)dropin_nfru();
}

static void die(const char *where, int rc)
{
    fprintf(stderr, "gw_fru: %s failed (%d): %s\n", where, rc, gw_last_error());
    abort();
}

static gw_ctx *need_ctx(const char *where)
{
    if (!g_ctx) {
        fprintf(stderr, "gw_fru: %s called before initialize_mpi_state\n", where);
        abort();
    }
    return g_ctx;
}

void initialize_mpi(int *argc, char **argv, int *rank, int *procs)
{
    (void)argc;
    (void)argv;
    *rank = 0;
    *procs = 1;
}

void end_mpi(void)
{
    if (g_ctx) gw_destroy(g_ctx);
    g_ctx = NULL;
}

void parallel(void) {}

void initialize_mpi_state(double FRU_states[][5], int LType_state[][4][2], int RyR_state[][4][5],
                          int Ito2_state[][4], int mti[], unsigned long mt[][625])
{
    const int n = dropin_nfru();
    uint32_t *w;
    int f, k, rc;
    if (g_ctx && gw_nfru(g_ctx) != n) end_mpi();
    if (!g_ctx && (rc = gw_create(&g_ctx, n))) die("initialize_mpi_state/gw_create", rc);
    gw_set_scale(g_ctx, dropin_scale());
    w = (uint32_t *)malloc(sizeof(uint32_t) * 624 * (size_t)n);
    if (!w) die("initialize_mpi_state/malloc", GW_ENOMEM);
    for (f = 0; f < n; f++)
        for (k = 0; k < 624; k++) w[(size_t)f * 624 + k] = (uint32_t)mt[f][k];
    rc = gw_upload(g_ctx, &FRU_states[0][0], &LType_state[0][0][0], &RyR_state[0][0][0], &Ito2_state[0][0], mti, w);
    free(w);
    if (rc) die("initialize_mpi_state/gw_upload", rc);
}

void distrib_simFRU(double st_time, double end_time, double FRUdep_states0[3], double FRUdep_statesf[3],
                    double *Jxfer, double *Jtr, double *ICa, double *Ito2)
{
    double J[4];
    int rc = gw_stage(need_ctx("distrib_simFRU"), st_time, end_time, FRUdep_states0, FRUdep_statesf, J, NULL);
    if (rc) die("distrib_simFRU", rc);
    *Jxfer = J[0];
    *Jtr = J[1];
    *ICa = J[2];
    *Ito2 = J[3];
}

void send_calc_fru_flux(double FRUdep_states[3], double *Jxfer, double *Jtr, double *ICa, double *Ito2)
{
    double J[4];
    int rc = gw_flux(need_ctx("send_calc_fru_flux"), FRUdep_states, J, NULL);
    if (rc) die("send_calc_fru_flux", rc);
    *Jxfer = J[0];
    *Jtr = J[1];
    *ICa = J[2];
    *Ito2 = J[3];
}

void send_calc_fru_avg(double state[37], double otherstate[12])
{
    double num[11];
    int rc = gw_avg_sums(need_ctx("send_calc_fru_avg"), num);
    if (rc) die("send_calc_fru_avg", rc);
    gw_otherstates(num, dropin_nfru(), dropin_scale(), state, otherstate);
}

void send_save_state(void)
{
    int rc = gw_save(need_ctx("send_save_state"));
    if (rc) die("send_save_state", rc);
}

void send_resume_state(void)
{
    int rc = gw_resume(need_ctx("send_resume_state"));
    if (rc) die("send_resume_state", rc);
}

void parallel_get_FRUs(double FRU_states[][5], int LType_state[][4][2], int RyR_state[][4][5], int Ito2_state[][4],
                       unsigned long mt[][625], int mti[])
{
    const int n = dropin_nfru();
    uint32_t *w = (uint32_t *)malloc(sizeof(uint32_t) * 624 * (size_t)n);
    int f, k, rc;
    if (!w) die("parallel_get_FRUs/malloc", GW_ENOMEM);
    rc = gw_download(need_ctx("parallel_get_FRUs"), &FRU_states[0][0], &LType_state[0][0][0], &RyR_state[0][0][0],
                     &Ito2_state[0][0], mti, w);
    if (rc) {
        free(w);
        die("parallel_get_FRUs", rc);
    }
    for (f = 0; f < n; f++)
        for (k = 0; k < 624; k++) mt[f][k] = w[(size_t)f * 624 + k];
    free(w);
}
