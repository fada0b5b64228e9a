/*
 * gw_caf -- C host driver of the GB300 FRU path: the reference program's main
 * loop (caf.c:43-285) on top of libgw_fru.so, with the run settings of
 * parameters.h read at run time instead of compiled in.
 *
 *   gw_caf [settings-file] [key=value ...]
 *
 * Settings file: one `key = value` per line, '#' starts a comment; keys are
 * the reference's parameters.h macro names (NFRU_sim, time_end, period,
 * vclamp_flag, ic_file_flag, ic_dir, output_dir, Ndump, ...) plus
 * seed_scheme (0: seed base+j, 1: initialize_ran.c formula) and seed_base.
 * Command-line key=value pairs override the file.
 *
 * Inputs and outputs keep the reference's formats byte for byte:
 * ic/stable/ic_*.txt (initialize_state.c:43-163, rewound every
 * min(NFRU,1250) FRUs), states.N.txt / otherstates.N.txt / currents.N.txt
 * (data_io.c:22-140), the r_*.N.txt checkpoint files (data_io.c:197-268)
 * every Ndump output steps, and with write_fru_props_flag = 1 the per-FRU
 * property files fruprops_J.N.txt, fruprops_avg_J.N.txt and
 * fruprops_avg_tot.N.txt for FRUs fru_start..fru_end (write_fru_props.c).
 *
 * Execution settings (not in the reference): precision = 0 (FP64, the
 * reference's arithmetic) or 1 (mixed: FP32 rates and local ODE),
 * fru_lanes = 4 or 1, stage_warps = 1/2/4/8 (warps per block) and
 * stage_packing = 0 or D (packed launches with 1/D as many warps as 8-FRU
 * groups); none of the shapes changes a result.  sum_order = 0 (one fixed
 * parallel order of the cross-FRU sums) or 1 (the serial reference's order,
 * a parity mode for small cells: with it the output files of an FP64 run
 * equal the reference program's byte for byte).
 *
 * Exact checkpoints (exact_restart = 1): beside the reference's r_*.N.txt
 * files, whose %g values cannot restart a run exactly, every checkpoint also
 * writes r_exact.N.bin with the full-precision global and FRU state, every
 * FRU's MT19937 words and position, the clock and the integrator's next step
 * size.  restart_file = <path> resumes from one: the resumed run writes the
 * same files, byte for byte, as the run that wrote the checkpoint went on to
 * write.  The file is native-endian (both supported hosts are little-endian):
 *   char magic[8] = "GWCKPT1"; int32 nfru, filenumber, iv_n, reserved;
 *   double time, oldstep, iv_time, state[37];
 *   double frus[n][5]; int32 ltype[n][4][2], ryr[n][4][5], ito2[n][4], mti[n];
 *   uint32 mt[n][624].
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gw_cell_model.h"
#include "gw_fru.h"

/* Host allocations: a run that cannot allocate stops with a message (the
 * reference aborts on its fatal errors too). */
static void *xmalloc(size_t bytes)
{
    void *p = malloc(bytes ? bytes : 1);
    if (!p) {
        fprintf(stderr, "gw_caf: out of host memory (%zu bytes)\n", bytes);
        exit(6);
    }
    return p;
}

static void *xcalloc(size_t n, size_t size)
{
    void *p = calloc(n ? n : 1, size ? size : 1);
    if (!p) {
        fprintf(stderr, "gw_caf: out of host memory (%zu x %zu bytes)\n", n, size);
        exit(6);
    }
    return p;
}

typedef struct {
    gw_settings s;
    int nfru, ts_sec, ic_file_flag, Ndump, filenumber0, seed_scheme;
    int write_fru_props_flag, fru_start, fru_end, fru_props_compat, exact_restart;
    int precision, fru_lanes, stage_warps, stage_packing, sum_order, reset_RyRs_flag;
    unsigned long seed_base;
    char ic_dir[512], output_dir[512], restart_file[512];
    char ic_states[128], ic_FRU[128], ic_LCh[128], ic_RyR[128], ic_Ito2[128];
} run_cfg;

static void cfg_defaults(run_cfg *c)
{
    memset(c, 0, sizeof *c);
    gw_settings_init(&c->s);
    c->nfru = 1000;            /* parameters.h:43-51 */
    c->ts_sec = 1;             /* parameters.h:101 */
    c->ic_file_flag = 1;       /* parameters.h:188 */
    c->Ndump = 10000;          /* parameters.h:209 */
    c->filenumber0 = 0;
    c->seed_scheme = 1;        /* the reference's initialize_ran.c formula */
    c->seed_base = 5489;
    c->fru_lanes = 4;
    c->stage_warps = 1;
    c->fru_start = 0;          /* parameters.h:203-205 */
    c->fru_end = 9;
    strcpy(c->ic_dir, "ic/stable");
    strcpy(c->output_dir, "./");
    strcpy(c->ic_states, "ic_states_stable.txt");
    strcpy(c->ic_FRU, "ic_FRU_stable.txt");
    strcpy(c->ic_LCh, "ic_LCh_stable.txt");
    strcpy(c->ic_RyR, "ic_RyR_stable.txt");
    strcpy(c->ic_Ito2, "ic_Ito2_stable.txt");
}

static char *trim(char *p)
{
    char *e;
    while (isspace((unsigned char)*p)) p++;
    e = p + strlen(p);
    while (e > p && isspace((unsigned char)e[-1])) *--e = 0;
    if (*p == '"' && e > p + 1 && e[-1] == '"') {
        e[-1] = 0;
        p++;
    }
    return p;
}

static int set_key(run_cfg *c, const char *k, const char *v)
{
#define DBL(name) if (!strcmp(k, #name)) { c->s.name = atof(v); return 0; }
#define INT(name) if (!strcmp(k, #name)) { c->s.name = atoi(v); return 0; }
    DBL(time_start) DBL(time_end) DBL(time_step) DBL(step_min) DBL(step_max) DBL(tolrk)
    DBL(pulse_duration) DBL(pulse_amplitude) DBL(period) DBL(shift)
    INT(vclamp_flag) DBL(vclamp_duration) DBL(vclamp_set) DBL(vclamp_shift) DBL(vclamp_hold) DBL(vclamp_period)
    INT(vppclamp_flag) DBL(vppclamp_ppset) DBL(vppclamp_ppduration) DBL(vppclamp_shift) DBL(vppclamp_set)
    DBL(vppclamp_duration) DBL(vppclamp_hold) DBL(vppclamp_period)
    INT(iv_flag) DBL(iv_clamp_duration) DBL(iv_clamp_period) DBL(iv_shift) DBL(iv_clamp_set) DBL(iv_clamp_hold)
    DBL(iv_clamp_step)
    INT(chf_flag) DBL(chfsc_IK1) DBL(chfsc_Jup) DBL(chfsc_INaCa) DBL(chfsc_IKv43) DBL(scale_PCa) DBL(scale_GKr)
#undef DBL
#undef INT
    if (!strcmp(k, "NFRU_sim") || !strcmp(k, "NFRU_sim_high") || !strcmp(k, "NFRU")) { c->nfru = atoi(v); return 0; }
    if (!strcmp(k, "ts_sec")) { c->ts_sec = atoi(v); return 0; }
    if (!strcmp(k, "ic_file_flag")) { c->ic_file_flag = atoi(v); return 0; }
    if (!strcmp(k, "reset_RyRs_flag")) { c->reset_RyRs_flag = atoi(v); return 0; }
    if (!strcmp(k, "Ndump")) { c->Ndump = atoi(v); return 0; }
    if (!strcmp(k, "filenumber0")) { c->filenumber0 = atoi(v); return 0; }
    if (!strcmp(k, "seed_scheme")) { c->seed_scheme = atoi(v); return 0; }
    if (!strcmp(k, "seed_base")) { c->seed_base = strtoul(v, NULL, 10); return 0; }
    if (!strcmp(k, "write_fru_props_flag")) { c->write_fru_props_flag = atoi(v); return 0; }
    if (!strcmp(k, "fru_start")) { c->fru_start = atoi(v); return 0; }
    if (!strcmp(k, "fru_end")) { c->fru_end = atoi(v); return 0; }
    if (!strcmp(k, "fru_props_compat")) { c->fru_props_compat = atoi(v); return 0; }
    if (!strcmp(k, "exact_restart")) { c->exact_restart = atoi(v); return 0; }
    if (!strcmp(k, "precision")) { c->precision = atoi(v); return 0; }
    if (!strcmp(k, "fru_lanes")) { c->fru_lanes = atoi(v); return 0; }
    if (!strcmp(k, "stage_warps")) { c->stage_warps = atoi(v); return 0; }
    if (!strcmp(k, "stage_packing")) { c->stage_packing = atoi(v); return 0; }
    if (!strcmp(k, "sum_order")) { c->sum_order = atoi(v); return 0; }
#define STR(field, name) if (!strcmp(k, name)) { snprintf(c->field, sizeof c->field, "%s", v); return 0; }
    STR(ic_dir, "ic_dir") STR(output_dir, "output_dir") STR(ic_states, "ic_states_file") STR(ic_FRU, "ic_FRU_file")
    STR(ic_LCh, "ic_LCh_file") STR(ic_RyR, "ic_RyR_file") STR(ic_Ito2, "ic_Ito2_file")
    STR(restart_file, "restart_file")
#undef STR
    return -1;
}

static int parse_line(run_cfg *c, char *line, const char *where)
{
    char *h = strchr(line, '#'), *eq, *k, *v;
    if (h) *h = 0;
    k = trim(line);
    if (!*k) return 0;
    eq = strchr(k, '=');
    if (!eq) {
        fprintf(stderr, "%s: expected key = value: '%s'\n", where, k);
        return -1;
    }
    *eq = 0;
    v = trim(eq + 1);
    k = trim(k);
    if (set_key(c, k, v)) {
        fprintf(stderr, "%s: unknown setting '%s'\n", where, k);
        return -1;
    }
    return 0;
}

/* ---- tolerant readers of the IC files (data_io.c:142-194) ---------------- */
static double read_next_double(FILE *f)
{
    char buf[256];
    int ch, i = 0;
    do ch = fgetc(f); while (ch != EOF && isspace(ch));
    while (ch != EOF && (isdigit(ch) || ch == 'E' || ch == 'e' || ch == '-' || ch == '+' || ch == '.') && i < 255) {
        buf[i++] = (char)ch;
        ch = fgetc(f);
    }
    buf[i] = 0;
    if (i < 1) {
        fprintf(stderr, "Error reading ic file: no decent input!\n");
        return 0;
    }
    return strtod(buf, NULL);
}

static int read_next_int(FILE *f)
{
    char buf[256];
    int ch, i = 0;
    do ch = fgetc(f); while (ch != EOF && isspace(ch));
    while (ch != EOF && (isdigit(ch) || ch == '-' || ch == '+') && i < 255) {
        buf[i++] = (char)ch;
        ch = fgetc(f);
    }
    buf[i] = 0;
    if (i < 1 || i > 30) {
        fprintf(stderr, "Error reading ic file: no decent input!\n");
        return 0;
    }
    return (int)strtol(buf, NULL, 10);
}

static FILE *open_ic(const run_cfg *c, const char *name)
{
    char path[1200];
    FILE *f;
    snprintf(path, sizeof path, "%s/%s", c->ic_dir, name);
    if (!(f = fopen(path, "rb"))) {
        fprintf(stderr, "Cannot open file '%s'!\n", path);
        exit(2);
    }
    return f;
}

/* FRU and global initial conditions from ic files (initialize_state.c:43-133),
 * each file rewound after every min(NFRU,1250) FRUs. */
static void read_ic(const run_cfg *c, double *state, double *frus, int *ltype, int *ryr, int *ito2)
{
    const int n = c->nfru, rw = n < 1250 ? n : 1250;
    FILE *f;
    int j, k;
    f = open_ic(c, c->ic_RyR);
    read_next_int(f);
    for (j = 0; j < n; j++) {
        for (k = 0; k < 20; k++) ryr[20 * j + k] = read_next_int(f);
        if ((j + 1) % rw == 0) { rewind(f); read_next_int(f); }
    }
    fclose(f);
    f = open_ic(c, c->ic_LCh);
    read_next_int(f);
    for (j = 0; j < n; j++) {
        for (k = 0; k < 8; k++) ltype[8 * j + k] = read_next_int(f);
        if ((j + 1) % rw == 0) { rewind(f); read_next_int(f); }
    }
    fclose(f);
    f = open_ic(c, c->ic_Ito2);
    read_next_int(f);
    for (j = 0; j < n; j++) {
        for (k = 0; k < 4; k++) ito2[4 * j + k] = read_next_int(f);
        if ((j + 1) % rw == 0) { rewind(f); read_next_int(f); }
    }
    fclose(f);
    f = open_ic(c, c->ic_FRU);
    read_next_int(f);
    for (j = 0; j < n; j++) {
        for (k = 0; k < 5; k++) frus[5 * j + k] = read_next_double(f);
        if ((j + 1) % rw == 0) { rewind(f); read_next_int(f); }
    }
    fclose(f);
    f = open_ic(c, c->ic_states);
    for (k = 0; k < GW_NSTATE; k++) state[k] = read_next_double(f);
    fclose(f);
}

/* ---- output files (data_io.c:22-140) ------------------------------------ */
static FILE *open_out(const run_cfg *c, const char *stem, int num)
{
    char path[1200];
    FILE *f;
    snprintf(path, sizeof path, "%s%s.%d.txt", c->output_dir, stem, num);
    if (!(f = fopen(path, "w+"))) {
        fprintf(stderr, "Cannot open file '%s'!\n", path);
        exit(3);
    }
    return f;
}

static FILE *open_states(const run_cfg *c, int num)
{
    FILE *f = open_out(c, "states", num);
    fprintf(f, "Time V mNa hNa jNa Nai Ki Cai CaNSR xKs LTRPNCa HTRPNCa C0Kv43 C1Kv43 C2Kv43 C3Kv43 OKv43 CI0Kv43 "
               "CI1Kv43 CI2Kv43 CI3Kv43 OIKv43 C0Kv14 C1Kv14 C2Kv14 C3Kv14 OKv14 CI0Kv14 CI1Kv14 CI2Kv14 CI3Kv14 "
               "OIKv14 CaToT C1Herg C2Herg C3Herg OHerg IHerg\n");
    return f;
}

static FILE *open_otherstates(const run_cfg *c, int num)
{
    FILE *f = open_out(c, "otherstates", num);
    fprintf(f, "Time CaSSavg CaJSRavg JRyRtot PRyR_open PRyR_ready PNorm_mode PnotVinact PLType_open CaToT2 "
               "PIto2_open CaJSRtot CaSStot \n");
    return f;
}

static FILE *open_currents(const run_cfg *c, int num)
{
    FILE *f = open_out(c, "currents", num);
    fprintf(f, "Time INa IKr IKs Ito1 IK1 IKp INaCa INaK IpCa ICab INab ICa JDHPR Jup Jtrpn Jtr Jxfer IKv43 IKv14 "
               "IKv14_K IKv14_Na Ito2 Istim Itot \n");
    return f;
}

static void write_row(FILE *f, const run_cfg *c, double t, const double *v, int n, const char *fmt)
{
    int i;
    fprintf(f, "%g ", c->ts_sec ? t * 1.e-3 : t);
    for (i = 0; i < n; i++) fprintf(f, fmt, v[i]);
    fprintf(f, "\n");
}

/* checkpoint files r_*.N.txt (data_io.c:197-268) */
static void restart_data(const run_cfg *c, int num, const double *state, gw_ctx *ctx)
{
    const int n = c->nfru;
    double *frus = xmalloc(sizeof(double) * 5 * n);
    int *ltype = xmalloc(sizeof(int) * 8 * n), *ryr = xmalloc(sizeof(int) * 20 * n), *ito2 = xmalloc(sizeof(int) * 4 * n);
    FILE *fs, *ff, *fl, *fr, *fi;
    int j, k, q;
    if (!frus || !ltype || !ryr || !ito2 || gw_download(ctx, frus, ltype, ryr, ito2, NULL, NULL)) {
        fprintf(stderr, "restart_data: download failed: %s\n", gw_last_error());
        exit(4);
    }
    fs = open_out(c, "r_states", num);
    for (k = 0; k < GW_NSTATE; k++) fprintf(fs, "%g\n", state[k]);
    ff = open_out(c, "r_FRU", num);
    fl = open_out(c, "r_LCh", num);
    fr = open_out(c, "r_RyR", num);
    fi = open_out(c, "r_Ito2", num);
    fprintf(ff, "%d\n", n);
    fprintf(fr, "%d\n", n);
    fprintf(fl, "%d\n", n);
    fprintf(fi, "%d\n", n);
    for (j = 0; j < n; j++) {
        for (k = 0; k < 5; k++) fprintf(ff, "%g ", frus[5 * j + k]);
        fprintf(ff, "\n");
        for (q = 0; q < 4; q++) {
            fprintf(fl, "%d %d\n", ltype[8 * j + 2 * q], ltype[8 * j + 2 * q + 1]);
            for (k = 0; k < 5; k++) fprintf(fr, "%d ", ryr[20 * j + 5 * q + k]);
            fprintf(fr, "\n");
            fprintf(fi, "%d\n", ito2[4 * j + q]);
        }
    }
    fclose(ff); fclose(fs); fclose(fr); fclose(fl); fclose(fi);
    free(frus); free(ltype); free(ryr); free(ito2);
}

/* ---- exact checkpoints ------------------------------------------------------ */
typedef struct {
    char magic[8];
    int32_t nfru, filenumber, iv_n, reserved;
    double time, oldstep, iv_time, state[GW_NSTATE];
} exact_header;

static const char kExactMagic[8] = "GWCKPT1";

static int write_all(FILE *f, const void *p, size_t size, size_t n) { return fwrite(p, size, n, f) == n ? 0 : -1; }
static int read_all(FILE *f, void *p, size_t size, size_t n) { return fread(p, size, n, f) == n ? 0 : -1; }

/* r_exact.<num>.bin: the state the run continues from, filenumber being the
 * number its next output files take */
static void write_exact(const run_cfg *c, int num, int filenumber, double time, double oldstep, double iv_time,
                        const double *state, gw_ctx *ctx)
{
    const int n = c->nfru;
    exact_header h;
    char path[1200];
    FILE *f;
    double *frus = xmalloc(sizeof(double) * 5 * n);
    int *ltype = xmalloc(sizeof(int) * 8 * n), *ryr = xmalloc(sizeof(int) * 20 * n), *ito2 = xmalloc(sizeof(int) * 4 * n);
    int *mti = xmalloc(sizeof(int) * n);
    uint32_t *mt = xmalloc(sizeof(uint32_t) * 624 * (size_t)n);
    int bad;
    if (!frus || !ltype || !ryr || !ito2 || !mti || !mt || gw_download(ctx, frus, ltype, ryr, ito2, mti, mt)) {
        fprintf(stderr, "exact checkpoint: download failed: %s\n", gw_last_error());
        exit(4);
    }
    memset(&h, 0, sizeof h);
    memcpy(h.magic, kExactMagic, 8);
    h.nfru = n;
    h.filenumber = filenumber;
    h.iv_n = c->s.iv_n;
    h.time = time;
    h.oldstep = oldstep;
    h.iv_time = iv_time;
    memcpy(h.state, state, sizeof h.state);
    snprintf(path, sizeof path, "%sr_exact.%d.bin", c->output_dir, num);
    if (!(f = fopen(path, "wb"))) {
        fprintf(stderr, "Cannot open file '%s'!\n", path);
        exit(3);
    }
    bad = write_all(f, &h, sizeof h, 1) || write_all(f, frus, sizeof(double), 5 * (size_t)n) ||
          write_all(f, ltype, sizeof(int), 8 * (size_t)n) || write_all(f, ryr, sizeof(int), 20 * (size_t)n) ||
          write_all(f, ito2, sizeof(int), 4 * (size_t)n) || write_all(f, mti, sizeof(int), (size_t)n) ||
          write_all(f, mt, sizeof(uint32_t), 624 * (size_t)n);
    if (fclose(f) || bad) {
        fprintf(stderr, "Cannot write file '%s'!\n", path);
        exit(3);
    }
    free(frus); free(ltype); free(ryr); free(ito2); free(mti); free(mt);
}

/* Resume from an exact checkpoint: uploads the FRU and MT state and returns
 * the clock, step size and file number the run continues with. */
static void read_exact(run_cfg *c, gw_ctx *ctx, double *state, double *time, double *oldstep, double *iv_time,
                       int *filenumber)
{
    const int n = c->nfru;
    exact_header h;
    FILE *f = fopen(c->restart_file, "rb");
    double *frus = xmalloc(sizeof(double) * 5 * n);
    int *ltype = xmalloc(sizeof(int) * 8 * n), *ryr = xmalloc(sizeof(int) * 20 * n), *ito2 = xmalloc(sizeof(int) * 4 * n);
    int *mti = xmalloc(sizeof(int) * n);
    uint32_t *mt = xmalloc(sizeof(uint32_t) * 624 * (size_t)n);
    if (!f) {
        fprintf(stderr, "Cannot open file '%s'!\n", c->restart_file);
        exit(2);
    }
    if (!frus || !ltype || !ryr || !ito2 || !mti || !mt) {
        fprintf(stderr, "restart: out of host memory\n");
        exit(4);
    }
    if (read_all(f, &h, sizeof h, 1) || memcmp(h.magic, kExactMagic, 8)) {
        fprintf(stderr, "'%s' is not an exact checkpoint\n", c->restart_file);
        exit(2);
    }
    if (h.nfru != n) {
        fprintf(stderr, "'%s' holds %d FRUs, the run has %d\n", c->restart_file, (int)h.nfru, n);
        exit(2);
    }
    if (read_all(f, frus, sizeof(double), 5 * (size_t)n) || read_all(f, ltype, sizeof(int), 8 * (size_t)n) ||
        read_all(f, ryr, sizeof(int), 20 * (size_t)n) || read_all(f, ito2, sizeof(int), 4 * (size_t)n) ||
        read_all(f, mti, sizeof(int), (size_t)n) || read_all(f, mt, sizeof(uint32_t), 624 * (size_t)n)) {
        fprintf(stderr, "'%s' is truncated\n", c->restart_file);
        exit(2);
    }
    fclose(f);
    if (gw_upload(ctx, frus, ltype, ryr, ito2, mti, mt)) {
        fprintf(stderr, "restart upload failed: %s\n", gw_last_error());
        exit(5);
    }
    memcpy(state, h.state, sizeof h.state);
    *time = h.time;
    *oldstep = h.oldstep;
    *iv_time = h.iv_time;
    *filenumber = h.filenumber;
    c->s.iv_n = h.iv_n;
    free(frus); free(ltype); free(ryr); free(ito2); free(mti); free(mt);
}

/* ---- per-FRU property files (write_fru_props.c:28-188) ------------------- */
typedef struct {
    FILE **fru, **avg, *tot;
    int n;                     /* fru_end - fru_start + 1 */
    double *frus;
    int *ltype, *ryr, *ito2;
} fru_props;

static void open_props(const run_cfg *c, int num, fru_props *p)
{
    char stem[64];
    int j;
    for (j = 0; j < p->n; j++) {
        snprintf(stem, sizeof stem, "fruprops_%d", c->fru_start + j);
        p->fru[j] = open_out(c, stem, num);
        fprintf(p->fru[j], "%s %s %s %s %s %s %s %s %s\n", "Time", "JLType", "JRyR", "Jtr", "Jxfer", "CaSS", "CaJSR",
                "Ito2", "NRyR_open");
    }
    for (j = 0; j < p->n; j++) {
        snprintf(stem, sizeof stem, "fruprops_avg_%d", c->fru_start + j);
        p->avg[j] = open_out(c, stem, num);
        fprintf(p->avg[j], "%s %s %s %s %s %s %s %s %s\n", "Time", "JLType_tot", "JRyR_tot", "Jtr", "Jxfer_tot",
                "CaSS_avg", "CaJSR", "Ito2", "PRyR_open");
    }
    p->tot = open_out(c, "fruprops_avg_tot", num);
    fprintf(p->tot, "%s %s %s %s %s %s %s %s %s\n", "Time", "JLType_totAll", "JRyR_totAll", "Jtr_totAll",
            "Jxfer_totAll", "CaSS_avgAll", "CaJSR_avgAll", "Ito2", "PRyR_openAll");
}

static void close_props(fru_props *p)
{
    int j;
    for (j = 0; j < p->n; j++) {
        fclose(p->fru[j]);
        fclose(p->avg[j]);
    }
    fclose(p->tot);
}

/* One output step of write_fru_props.c:28-128: only the selected FRUs are
 * read back from the device.  The reference tests an FRU's LCC as
 * LType_state[j][index_LCC_states][jcleft] and its voltage gate as
 * LType_state[j][index_LCC_Vinact][jcleft] (write_fru_props.c:90-91), with
 * the cleft and state subscripts swapped; this writes the LCC flux of the
 * cleft's own channel, or with fru_props_compat = 1 reads the same words of
 * the FRU's row as that code does (row offsets jcleft and 2 + jcleft). */
static void write_props(const run_cfg *c, fru_props *p, gw_ctx *ctx, double time, const double *state)
{
    const double V = state[GW_V], Cai = state[GW_Cai], CaNSR = state[GW_CaNSR];
    const double tprint = c->ts_sec ? time * 1.e-3 : time;
    const double VF_over_RT = V / GWC_RT_over_F, VFsq_over_RT = (1000.0 * GWC_Faraday) * VF_over_RT;
    const double pca = GWC_PCa * c->s.scale_PCa;
    double JLType_totALL = 0.0, JRyR_totALL = 0.0, Jtr_totALL = 0.0, Jxfer_totALL = 0.0;
    double CaSS_avgALL = 0.0, CaJSR_avgALL = 0.0, PRyR_openALL = 0.0, Ito2_avgALL = 0.0, num_avg;
    int j, q, i;
    if (gw_download_range(ctx, c->fru_start, p->n, p->frus, p->ltype, p->ryr, p->ito2)) {
        fprintf(stderr, "write_fru_props: download failed: %s\n", gw_last_error());
        exit(4);
    }
    for (j = 0; j < p->n; j++) {
        const double CaJSR = p->frus[5 * j];
        const int *lt = p->ltype + 8 * j;
        double JLType_tot1 = 0.0, JRyR_tot1 = 0.0, Jxfer_tot1 = 0.0, CaSS_avg1 = 0.0, PRyR_open1 = 0.0;
        double Ito2_tot1 = 0.0, Jtr;
        CaJSR_avgALL = CaJSR_avgALL + CaJSR;
        Jtr = (CaNSR - CaJSR) / GWC_tautr * GWC_VJSR / GWC_Vmyo;
        Jtr_totALL = Jtr_totALL + Jtr;
        for (q = 0; q < 4; q++) {
            const double CaSS = p->frus[5 * j + q + 1];
            const int lcc = c->fru_props_compat ? lt[q] : lt[2 * q];
            const int vdi = c->fru_props_compat ? lt[2 + q] : lt[2 * q + 1];
            double JLType = 0.0, Ito2 = 0.0, JRyR, Jxfer;
            int nopen = 0;
            CaSS_avg1 += CaSS;
            CaSS_avgALL += CaSS;
            if ((lcc == 6 || lcc == 12) && vdi == 2) { /* O1_LType, O2_LType, Oy_LType */
                JLType = pca * 4.0 * VFsq_over_RT * (CaSS * exp(2.0 * VF_over_RT) - GWC_Cao * 0.341) /
                         (exp(2.0 * VF_over_RT) - 1.0) / (-2.0 * GWC_Vmyo * GWC_Faraday * 1000.0);
                JLType_tot1 += JLType;
                JLType_totALL += JLType;
            }
            if (p->ito2[4 * j + q] == 2) { /* O_Ito2 */
                Ito2 = GWC_PCl * VFsq_over_RT * (GWC_Cli * exp(-VF_over_RT) - GWC_Clo) / (exp(-VF_over_RT) - 1.0);
                Ito2_tot1 += Ito2;
                Ito2_avgALL += Ito2;
            }
            for (i = 0; i < 5; i++) {
                const int r = p->ryr[20 * j + 5 * q + i];
                if (r == 3 || r == 4 || r == 7) nopen = nopen + 1; /* O1_RyR, O2_RyR, O3_RyR */
            }
            PRyR_open1 = PRyR_open1 + (double)nopen;
            PRyR_openALL = PRyR_openALL + (double)nopen;
            JRyR = GWC_JRyRmax * (double)nopen * (CaJSR - CaSS) * GWC_VSS / GWC_Vmyo;
            JRyR_tot1 = JRyR_tot1 + JRyR;
            JRyR_totALL = JRyR_totALL + JRyR;
            Jxfer = (CaSS - Cai) / GWC_tauxfer * GWC_VSS / GWC_Vmyo;
            Jxfer_tot1 = Jxfer_tot1 + Jxfer;
            Jxfer_totALL = Jxfer_totALL + Jxfer;
            fprintf(p->fru[j], "%.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %d\n", tprint, JLType, JRyR, Jtr, Jxfer, CaSS,
                    CaJSR, Ito2, nopen);
        }
        CaSS_avg1 = CaSS_avg1 / 4;
        PRyR_open1 = PRyR_open1 / (double)(5 * 4);
        fprintf(p->avg[j], "%.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g\n", tprint, JLType_tot1, JRyR_tot1, Jtr,
                Jxfer_tot1, CaSS_avg1, CaJSR, Ito2_tot1, PRyR_open1);
    }
    num_avg = (double)p->n;
    CaSS_avgALL = CaSS_avgALL / num_avg / 4;
    CaJSR_avgALL = CaJSR_avgALL / num_avg;
    PRyR_openALL = PRyR_openALL / (num_avg * (double)(5 * 4));
    fprintf(p->tot, "%.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g\n", tprint, JLType_totALL, JRyR_totALL, Jtr_totALL,
            Jxfer_totALL, CaSS_avgALL, CaJSR_avgALL, Ito2_avgALL, PRyR_openALL);
}

/* initial conditions (initialize_ran.c + initialize_state.c) */
static void init_cell(const run_cfg *c, gw_ctx *ctx, double *state)
{
    const int n = c->nfru;
    if (!c->ic_file_flag) {
        if (gw_init_rest(ctx, &c->s, c->seed_scheme, (uint32_t)c->seed_base, state)) {
            fprintf(stderr, "gw_init_rest: %s\n", gw_last_error());
            exit(5);
        }
        return;
    }
    {
        double *frus = xmalloc(sizeof(double) * 5 * n), a1 = 0.0, a2 = 0.0;
        int *ltype = xmalloc(sizeof(int) * 8 * n), *ryr = xmalloc(sizeof(int) * 20 * n);
        int *ito2 = xmalloc(sizeof(int) * 4 * n), *mti = xmalloc(sizeof(int) * n), j, q, k;
        uint32_t *mt = xcalloc((size_t)624 * n, sizeof(uint32_t));
        read_ic(c, state, frus, ltype, ryr, ito2);
        if (c->reset_RyRs_flag)  /* initialize_state.c:252-263: every LCC closed and available, every RyR in 1 */
            for (j = 0; j < n; j++)
                for (q = 0; q < 4; q++) {
                    ltype[8 * j + 2 * q] = 1;
                    ltype[8 * j + 2 * q + 1] = 2;
                    for (k = 0; k < 5; k++) ryr[20 * j + 5 * q + k] = 1;
                }
        for (j = 0; j < n; j++) mti[j] = 624;
        if (gw_upload(ctx, frus, ltype, ryr, ito2, mti, mt) || gw_seed(ctx, c->seed_scheme, (uint32_t)c->seed_base)) {
            fprintf(stderr, "initial upload failed: %s\n", gw_last_error());
            exit(5);
        }
        if (c->s.vclamp_flag) state[GW_V] = c->s.vclamp_hold;
        if (c->s.iv_flag) state[GW_V] = c->s.iv_clamp_hold;
        for (j = 0; j < n; j++) {
            a1 = a1 + frus[5 * j] * (1.0 + GWC_CSQNtot / (GWC_KmCSQN + frus[5 * j]));
            for (q = 0; q < 4; q++)
                a2 = a2 + frus[5 * j + q + 1] * (1.0 + GWC_BSRtot / (GWC_KBSR + frus[5 * j + q + 1]) +
                                                  GWC_BSLtot / (GWC_KBSL + frus[5 * j + q + 1]));
        }
        state[GW_CaTOT] = gw_catot(a1, a2, 12500.0 / n, state);
        if (c->s.vclamp_flag) state[GW_V] = c->s.vclamp_hold;
        free(frus); free(ltype); free(ryr); free(ito2); free(mti); free(mt);
    }
}

int main(int argc, char **argv)
{
    run_cfg c;
    gw_ctx *ctx = NULL;
    double state[GW_NSTATE], cur[GW_NCUR], other[GW_NOTHER], num[11];
    double time_now, tstep, oldstep, iv_time = 0.0;
    int filenumber, n_restart = 0, a, rc;
    FILE *fst, *fcu, *fot;
    fru_props props;
    clock_t c0 = clock();

    cfg_defaults(&c);
    for (a = 1; a < argc; a++) {
        if (strchr(argv[a], '=')) {
            char buf[1024];
            snprintf(buf, sizeof buf, "%s", argv[a]);
            if (parse_line(&c, buf, "command line")) return 1;
        } else {
            FILE *f = fopen(argv[a], "r");
            char line[1024];
            if (!f) {
                fprintf(stderr, "Cannot open settings file '%s'\n", argv[a]);
                return 1;
            }
            while (fgets(line, sizeof line, f))
                if (parse_line(&c, line, argv[a])) return 1;
            fclose(f);
        }
    }
    if ((rc = gw_create(&ctx, c.nfru))) {
        fprintf(stderr, "gw_create: %s\n", gw_last_error());
        return 1;
    }
    gw_set_scale(ctx, 12500.0 / c.nfru);
    if (gw_set_precision(ctx, c.precision) || gw_set_fru_lanes(ctx, c.fru_lanes) ||
        gw_set_stage_warps(ctx, c.stage_warps) || gw_set_pca_scale(ctx, c.s.scale_PCa) ||
        gw_set_sum_order(ctx, c.sum_order) ||
        gw_set_stage_packing(ctx, c.stage_packing > 0 ? ((c.nfru + 7) / 8 + c.stage_packing - 1) / c.stage_packing : 0)) {
        fprintf(stderr, "execution settings: %s\n", gw_last_error());
        return 1;
    }
    oldstep = c.s.step_max;
    filenumber = c.filenumber0;
    if (c.restart_file[0])
        read_exact(&c, ctx, state, &c.s.time_start, &oldstep, &iv_time, &filenumber);
    else
        init_cell(&c, ctx, state);
    fst = open_states(&c, filenumber);
    fcu = open_currents(&c, filenumber);
    fot = open_otherstates(&c, filenumber);
    memset(&props, 0, sizeof props);
    if (c.write_fru_props_flag) {
        if (c.fru_end >= c.nfru) { /* write_fru_props.c:60-68 */
            fprintf(stderr, "Inappropriate fru_end (%d) in write_fru_props\n", c.fru_end);
            exit(-3);
        }
        if (c.fru_start < 0 || c.fru_start > c.fru_end) {
            fprintf(stderr, "Inappropriate fru_start (%d) in write_fru_props\n", c.fru_start);
            exit(-4);
        }
        props.n = c.fru_end - c.fru_start + 1;
        props.fru = xmalloc(sizeof(FILE *) * props.n);
        props.avg = xmalloc(sizeof(FILE *) * props.n);
        props.frus = xmalloc(sizeof(double) * 5 * props.n);
        props.ltype = xmalloc(sizeof(int) * 8 * props.n);
        props.ryr = xmalloc(sizeof(int) * 20 * props.n);
        props.ito2 = xmalloc(sizeof(int) * 4 * props.n);
        if (!props.fru || !props.avg || !props.frus || !props.ltype || !props.ryr || !props.ito2) {
            fprintf(stderr, "write_fru_props: out of host memory\n");
            exit(4);
        }
        open_props(&c, filenumber, &props);
    }
    printf("%s %s %s %s\n", "Time", "Phase", "NFRU", "V");
    for (time_now = c.s.time_start; time_now <= c.s.time_end - .0001 * c.s.time_step; time_now += c.s.time_step) {
        printf("%g %i %i %g\n", time_now, 1, c.nfru, state[GW_V]);
        n_restart = n_restart + 1;
        tstep = time_now + c.s.time_step;
        iv_time = iv_time + c.s.time_step;
        if ((rc = gw_rk54pd(ctx, &c.s, time_now, tstep, oldstep, state, cur, &oldstep)) ||
            (rc = gw_avg_sums(ctx, num))) {
            fprintf(stderr, "step at t=%g failed: %s\n", time_now, gw_last_error());
            return 1;
        }
        gw_otherstates(num, c.nfru, 12500.0 / c.nfru, state, other);
        if (time_now > c.s.time_start) {
            if (n_restart == 1) {
                fclose(fcu);
                fcu = open_currents(&c, filenumber);
            } else {
                write_row(fcu, &c, time_now, cur, GW_NCUR, "%g ");
            }
        }
        write_row(fst, &c, tstep, state, GW_NSTATE, "%.8g ");
        write_row(fot, &c, tstep, other, GW_NOTHER, "%g ");
        if (c.write_fru_props_flag) write_props(&c, &props, ctx, tstep, state);
        if (n_restart >= c.Ndump) {
            n_restart = 0;
            restart_data(&c, filenumber, state, ctx);
            if (c.exact_restart) write_exact(&c, filenumber, filenumber + 1, tstep, oldstep, iv_time, state, ctx);
            filenumber = filenumber + 1;
            fclose(fot);
            fclose(fst);
            if (c.write_fru_props_flag) close_props(&props);
            if (time_now < c.s.time_end - 1.0001 * c.s.time_step) {
                fst = open_states(&c, filenumber);
                fot = open_otherstates(&c, filenumber);
                if (c.write_fru_props_flag) open_props(&c, filenumber, &props);
            } else {
                fst = fot = NULL;
                props.tot = NULL;
            }
        }
        if (c.s.iv_flag && iv_time >= c.s.iv_clamp_period) {
            iv_time = 0.0;
            c.s.iv_n = c.s.iv_n + 1;
            oldstep = c.s.step_max;
            init_cell(&c, ctx, state);
        }
    }
    if ((rc = gw_lastcall(ctx, &c.s, c.s.time_end, state, cur))) {
        fprintf(stderr, "lastcall failed: %s\n", gw_last_error());
        return 1;
    }
    write_row(fcu, &c, c.s.time_end, cur, GW_NCUR, "%g ");
    fclose(fcu);
    if (fot) fclose(fot);
    if (fst) fclose(fst);
    if (c.write_fru_props_flag && props.tot) close_props(&props);
    gw_destroy(ctx);
    printf("Total time: %fs\n", (double)(clock() - c0) / (double)CLOCKS_PER_SEC);
    return 0;
}
