/*
 * Test-only stand-in for the GPU half of libgw_fru.so: the native gw_* FRU
 * operations implemented on the CPU oracle (oracle/fru_oracle.c).  Linked with
 * the product's host sources (gw_dp.c, gw_dropin.c) it lets the CPU test suite
 * run the product's Dormand-Prince driver and drop-in layer end to end and
 * compare them with the reference build.  Never part of the product.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gw_fru.h"

void orc_sgrnd(uint32_t seed, int *mti, uint32_t mt[624]);
void orc_seed_reference_all(int n, uint32_t *seeds);
void orc_simfru_batch(int n, double t0, double tf, const double dep0[3], const double depf[3], int *ltype,
                      int *ryr, int *ito2, double *frus, int *mti, uint32_t *mt);
void orc_flux_sums(int n, const int *ltype, const int *ito2, const double *frus, double num[5]);
void orc_avg_sums(int n, const int *ltype, const int *ryr, const int *ito2, const double *frus, double num[11]);
void orc_currents(int nfru, double scale, const double dep[3], const double num[5], double out[4]);
unsigned long long orc_substep_count(void);

typedef struct {
    double *frus; int *ltype, *ryr, *ito2, *mti; uint32_t *mt;
} set_t;

struct gw_ctx {
    int n;
    double scale;
    set_t live, saved;
    unsigned long long substeps;
};

static int alloc_set(set_t *s, int n)
{
    s->frus = calloc((size_t)n * 5, sizeof(double));
    s->ltype = calloc((size_t)n * 8, sizeof(int));
    s->ryr = calloc((size_t)n * 20, sizeof(int));
    s->ito2 = calloc((size_t)n * 4, sizeof(int));
    s->mti = calloc((size_t)n, sizeof(int));
    s->mt = calloc((size_t)n * 624, sizeof(uint32_t));
    return s->frus && s->ltype && s->ryr && s->ito2 && s->mti && s->mt ? 0 : GW_ENOMEM;
}
static void free_set(set_t *s)
{
    free(s->frus); free(s->ltype); free(s->ryr); free(s->ito2); free(s->mti); free(s->mt);
}
/* NULL destination arrays are skipped (gw_download's optional outputs) */
static void copy_set(set_t *d, const set_t *s, int n)
{
    if (d->frus) memcpy(d->frus, s->frus, sizeof(double) * 5 * n);
    if (d->ltype) memcpy(d->ltype, s->ltype, sizeof(int) * 8 * n);
    if (d->ryr) memcpy(d->ryr, s->ryr, sizeof(int) * 20 * n);
    if (d->ito2) memcpy(d->ito2, s->ito2, sizeof(int) * 4 * n);
    if (d->mti) memcpy(d->mti, s->mti, sizeof(int) * n);
    if (d->mt) memcpy(d->mt, s->mt, sizeof(uint32_t) * 624 * n);
}

static char g_err[256] = "cpu test stand-in";
const char *gw_last_error(void) { return g_err; }
int gw_internal_error(int code, const char *msg)
{
    snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}
int gw_create(gw_ctx **out, int n)
{
    gw_ctx *c = calloc(1, sizeof *c);
    if (!c || n <= 0) return GW_EINVAL;
    c->n = n;
    c->scale = 12500.0 / n;
    if (alloc_set(&c->live, n) || alloc_set(&c->saved, n)) return GW_ENOMEM;
    *out = c;
    return GW_OK;
}
int gw_destroy(gw_ctx *c)
{
    if (c) { free_set(&c->live); free_set(&c->saved); free(c); }
    return GW_OK;
}
int gw_nfru(const gw_ctx *c) { return c ? c->n : 0; }
int gw_set_scale(gw_ctx *c, double s) { c->scale = s; return GW_OK; }
int gw_sync(gw_ctx *c) { (void)c; return GW_OK; }
int gw_upload(gw_ctx *c, const double *frus, const int *ltype, const int *ryr, const int *ito2, const int *mti,
              const uint32_t *mt)
{
    set_t src = {(double *)frus, (int *)ltype, (int *)ryr, (int *)ito2, (int *)mti, (uint32_t *)mt};
    copy_set(&c->live, &src, c->n);
    return GW_OK;
}
int gw_download(gw_ctx *c, double *frus, int *ltype, int *ryr, int *ito2, int *mti, uint32_t *mt)
{
    set_t dst = {frus, ltype, ryr, ito2, mti, mt};
    copy_set(&dst, &c->live, c->n);
    return GW_OK;
}
int gw_download_range(gw_ctx *c, int first, int count, double *frus, int *ltype, int *ryr, int *ito2)
{
    set_t src = {c->live.frus + 5 * first, c->live.ltype + 8 * first, c->live.ryr + 20 * first,
                 c->live.ito2 + 4 * first, NULL, NULL};
    set_t dst = {frus, ltype, ryr, ito2, NULL, NULL};
    if (first < 0 || count <= 0 || first + count > c->n) return GW_EINVAL;
    copy_set(&dst, &src, count);
    return GW_OK;
}
int gw_seed(gw_ctx *c, int scheme, uint32_t base)
{
    uint32_t *seeds = malloc(sizeof(uint32_t) * c->n);
    int j;
    if (scheme == 1) orc_seed_reference_all(c->n, seeds);
    else for (j = 0; j < c->n; j++) seeds[j] = base + (uint32_t)j;
    for (j = 0; j < c->n; j++) orc_sgrnd(seeds[j], &c->live.mti[j], c->live.mt + (size_t)624 * j);
    free(seeds);
    return GW_OK;
}
int gw_stage(gw_ctx *c, double t0, double tf, const double dep0[3], const double depf[3], double out[4],
             double num[5])
{
    double nm[5];
    set_t *s = &c->live;
    static int nstage = 0;
    const unsigned long long before = orc_substep_count();
    orc_simfru_batch(c->n, t0, tf, dep0, depf, s->ltype, s->ryr, s->ito2, s->frus, s->mti, s->mt);
    c->substeps += orc_substep_count() - before;
    /* GW_CPU_STAGE_LOG: one line per stage with its FRU-substeps, to pair
     * the stage launches of a GPU profile with their workload */
    if (getenv("GW_CPU_STAGE_LOG"))
        fprintf(stderr, "stage %d [%.6f, %.6f] FRU-substeps %llu\n", ++nstage, t0, tf,
                orc_substep_count() - before);
    orc_flux_sums(c->n, s->ltype, s->ito2, s->frus, nm);
    if (out) orc_currents(c->n, c->scale, depf, nm, out);
    if (num) memcpy(num, nm, sizeof nm);
    return GW_OK;
}
int gw_flux(gw_ctx *c, const double dep[3], double out[4], double num[5])
{
    double nm[5];
    orc_flux_sums(c->n, c->live.ltype, c->live.ito2, c->live.frus, nm);
    if (out) orc_currents(c->n, c->scale, dep, nm, out);
    if (num) memcpy(num, nm, sizeof nm);
    return GW_OK;
}
int gw_avg_sums(gw_ctx *c, double num[11])
{
    orc_avg_sums(c->n, c->live.ltype, c->live.ryr, c->live.ito2, c->live.frus, num);
    return GW_OK;
}
int gw_save(gw_ctx *c) { copy_set(&c->saved, &c->live, c->n); return GW_OK; }
int gw_resume(gw_ctx *c) { copy_set(&c->live, &c->saved, c->n); return GW_OK; }
int gw_substeps(gw_ctx *c, unsigned long long *n) { *n = c->substeps; return GW_OK; }
/* launch-shape and precision settings: the stand-in has one shape and FP64 only */
int gw_set_fru_lanes(gw_ctx *c, int lanes) { (void)c; return lanes == 1 || lanes == 4 ? GW_OK : GW_EINVAL; }
int gw_set_stage_warps(gw_ctx *c, int warps) { (void)c; return warps >= 1 && warps <= 8 ? GW_OK : GW_EINVAL; }
int gw_set_stage_packing(gw_ctx *c, int warps) { (void)c; return warps >= 0 ? GW_OK : GW_EINVAL; }
int gw_set_precision(gw_ctx *c, int precision) { (void)c; return precision == 0 ? GW_OK : GW_EINVAL; }
int gw_set_pca_scale(gw_ctx *c, double scale) { (void)c; return scale == 1.0 ? GW_OK : GW_EINVAL; }
/* the oracle's sums are always in the reference's order */
int gw_set_sum_order(gw_ctx *c, int order) { (void)c; return order == 0 || order == 1 ? GW_OK : GW_EINVAL; }
