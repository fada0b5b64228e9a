/*
 * CPU oracle for the FRU hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-FRU Monte Carlo, written for
 * checking the CUDA path.  Only tests/, the smoke check and the CPU-baseline
 * leg of bench.py may load it; the product never links it.
 *
 * Parity pin: tests/test_oracle.py compares every function here against the
 * reference itself (compiled from its own sources into oracle/_ref by
 * oracle/build_ref.py) and against the committed fixtures in tests/golden/.
 *
 * Floating point: every expression keeps the reference's operand order and
 * association, and this file is compiled with -ffp-contract=off, so results
 * are bit-identical to the reference build wherever libm's exp() agrees.
 *
 * Packed per-FRU layout (same as the reference's per-FRU arrays):
 *   ltype[4][2]  (LCC state 1..12, VDI gate 1..2)      parameters.h:30-40
 *   ryr[4][5]    (RyR state 1..8)
 *   ito2[4]      (Ca-activated Cl channel 1=closed, 2=open)
 *   frus[5]      (CaJSR, CaSS1..4)                      indices.h:81-88
 *   mti, mt[624] (MT19937 position and state words)     mt19937_local.c:76
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NCLEFT 4
#define NRYR 5
#define MTN 624
#define MTM 397

/* ---- physical constants: parameters_fcn_fru.c:21-90 ---------------------- */
static const double Cao = 2.0, Clo = 150.0, Cli = 20.0;
static const double Faraday = 96.5;
static const double RT_over_F = 8.314 * 310.0 / 96.5;
static const double Acap = 1.534e-4;
static const double VJSR = (((double)NCLEFT) * 0.53 * 0.5 * 0.2 * 1.05e-10);
static const double VSS = (0.5 * 0.2 * 2.03e-12);
static const double PCa = (1.5 / 2.8 * 0.2 * 0.9 * 0.9468e-11);
static const double PCl = 2.65e-15;
static const double BSLtot = 1.124, CSQNtot = 13.5, BSRtot = 0.047;
static const double KBSL = 0.0087, KmCSQN = 0.63, KBSR = 0.00087;
static const double JRyRmax = (0.6 * 1.5 * 1.1 * 3.96);
static const double tautr = 3.0, tauxfer = 0.005, tauss2ss = (10.0 * 0.005);

/* ---- MT19937 (mt19937_local.c:59-240; Matsumoto & Nishimura 1998) --------- */
void orc_sgrnd(uint32_t seed, int *mti, uint32_t mt[MTN])
{
    /* Knuth TAOCP vol.2 initialisation, mt19937_local.c:76-92 */
    uint32_t i;
    mt[0] = seed;
    for (i = 1; i < MTN; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i;
    *mti = MTN;
}

static void mt_regenerate(uint32_t mt[MTN])
{
    int k;
    for (k = 0; k < MTN; k++) {
        uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % MTN] & 0x7fffffffu);
        mt[k] = mt[(k + MTM) % MTN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
}

uint32_t orc_next_word(int *mti, uint32_t mt[MTN])
{
    uint32_t y;
    if (*mti >= MTN) { mt_regenerate(mt); *mti = 0; }
    y = mt[(*mti)++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double orc_next(int *mti, uint32_t mt[MTN])
{
    return ((double)orc_next_word(mti, mt)) / 4294967296.0;
}

/* Seed of FRU j in the reference (initialize_ran.c:30-34): a running int
 * a += 23*j, seed = abs(a + 4093*j*j) + 1, evaluated with 32-bit
 * two's-complement wrap-around (what the reference's int arithmetic does). */
uint32_t orc_seed_reference(int j)
{
    uint32_t a = 12350232u, t;
    int32_t s;
    int i;
    for (i = 0; i <= j; i++) a = a + 23u * (uint32_t)i;
    t = a + (4093u * (uint32_t)j) * (uint32_t)j;
    s = (int32_t)t;
    if (s < 0) s = (int32_t)(0u - (uint32_t)s);
    return (uint32_t)s + 1u;
}

/* Seeds of FRUs 0..n-1 by initialize_ran.c:30-34 (one pass). */
void orc_seed_reference_all(int n, uint32_t *seeds)
{
    uint32_t a = 12350232u, t;
    int32_t s;
    int j;
    for (j = 0; j < n; j++) {
        a = a + 23u * (uint32_t)j;
        t = a + (4093u * (uint32_t)j) * (uint32_t)j;
        s = (int32_t)t;
        if (s < 0) s = (int32_t)(0u - (uint32_t)s);
        seeds[j] = (uint32_t)s + 1u;
    }
}

/* ---- channel rates: fru_rates_local.c:30-798 ------------------------------ */
/* LCC modal gating constants, fru_rates_local.c:50-86 */
static const double fL = 0.85, gL = 2.0, fLprime = 0.005, gLprime = 7.0;
static const double bL = 1.9356, aL = 2.0;
#define bL2 (bL * bL)
#define bL3 (bL * bL * bL)
#define bL4 (bL * bL * bL * bL)
#define aL2 (aL * aL)
#define aL3 (aL * aL * aL)
#define aL4 (aL * aL * aL * aL)
static const double kappa = 1;
static const double omega = 0.83 * 2.0 * 1.3 * 0.01;
static const double alphacf = 4.0 * 1.2 * 0.416;
static const double betacf = 4.0 * 0.45 * 0.049;
static const double gammacf = 0.83 * 1.9 * 1.3 * 0.31 * 7.5 * 0.09233;
/* Ca-activated Cl channel, :94-96 */
static const double kbIto2 = 2.0;
#define kfIto2 (2.0 / 0.1502)
/* RyR, :100-121 */
static const double k21 = 250.0, k32 = 9.6, k43 = 0.07 / 0.06667 * 13.0, k45 = 0.07;
static const double k52 = 0.001235, k65 = 30.0;
static const double k12cf = 3000.0, k23cf = 10.0 * 30000.0, k34cf = 0.6 * 3000.0;
static const double k54cf = 0.6 * 0.198, k25cf = 10.0 * 300.0, k56cf = 2.0 * 4.0 * 3000.0;
static const double k_rate = 0.00127215, k_rate2 = 3.4188;
static const double threshCa34to7 = 0.0368369379834969;
static const double threshCa56to8 = 0.00011447933531005;
static const double threshMAX = 2.0, threshMAXCa = 0.0504410547074504;

#define DMIN(a, b) ((a) < (b) ? (a) : (b))
#define DMAX(a, b) ((a) < (b) ? (b) : (a))

/* One channel's exit table: total[0] and up to 3 (rate, destination) pairs. */
typedef struct { double r[4]; int dest[4]; int len; } exit_row;

static void row2(exit_row *e, double r1, int d1)
{
    e->r[0] = r1; e->r[1] = r1; e->dest[1] = d1; e->len = 2;
}
static void row3(exit_row *e, double tot, double r1, int d1, double r2, int d2)
{
    e->r[0] = tot; e->r[1] = r1; e->dest[1] = d1; e->r[2] = r2; e->dest[2] = d2; e->len = 3;
}
static void row4(exit_row *e, double tot, double r1, int d1, double r2, int d2, double r3, int d3)
{
    e->r[0] = tot; e->r[1] = r1; e->dest[1] = d1; e->r[2] = r2; e->dest[2] = d2;
    e->r[3] = r3; e->dest[3] = d3; e->len = 4;
}

/* LCC exit row for state s (fru_rates_local.c:176-340).  The totals keep the
 * reference's summation order, which differs from the row order in the
 * Ca-mode states 8..10. */
static void lcc_row(exit_row *e, int s, double alpha, double beta, double gam)
{
    double ap = aL * alpha, bp = beta / (bL * kappa);
    double r1, r2, r3;
    switch (s) {
    case 1: r1 = 4.0 * alpha; r2 = gam; row3(e, r1 + r2, r1, 2, r2, 7); break;
    case 2: r1 = beta; r2 = 3.0 * alpha; r3 = aL * gam; row4(e, r1 + r2 + r3, r1, 1, r2, 3, r3, 8); break;
    case 3: r1 = 2.0 * beta; r2 = 2.0 * alpha; r3 = aL2 * gam; row4(e, r1 + r2 + r3, r1, 2, r2, 4, r3, 9); break;
    case 4: r1 = 3.0 * beta; r2 = alpha; r3 = aL3 * gam; row4(e, r1 + r2 + r3, r1, 3, r2, 5, r3, 10); break;
    case 5: r1 = 4.0 * beta; r2 = fL; r3 = aL4 * gam; row4(e, r1 + r2 + r3, r1, 4, r2, 6, r3, 11); break;
    case 6: row2(e, gL, 5); break;
    case 7: r1 = kappa * kappa * kappa * kappa * omega; r2 = 4.0 * ap; row3(e, r2 + r1, r1, 1, r2, 8); break;
    case 8: r1 = bp; r2 = kappa * kappa * kappa * omega / bL; r3 = 3.0 * ap;
        row4(e, r1 + r3 + r2, r1, 7, r2, 2, r3, 9); break;
    case 9: r1 = 2.0 * bp; r2 = kappa * kappa * omega / bL2; r3 = 2.0 * ap;
        row4(e, r1 + r3 + r2, r1, 8, r2, 3, r3, 10); break;
    case 10: r1 = 3.0 * bp; r2 = kappa * omega / bL3; r3 = ap;
        row4(e, r1 + r3 + r2, r1, 9, r2, 4, r3, 11); break;
    case 11: r1 = 4.0 * bp; r2 = omega / bL4; r3 = fLprime; row4(e, r1 + r2 + r3, r1, 10, r2, 5, r3, 12); break;
    case 12: row2(e, gLprime, 11); break;
    default: e->r[0] = 0.0; e->len = 1; break; /* unknown state: reference prints and leaves stale rates */
    }
}

/* Per-cleft RyR rate constants (fru_rates_local.c:375-382). */
typedef struct { double k12, k23, k34, k54, k25, k56; int regime; } ryr_k;

static void ryr_constants(ryr_k *k, double cass)
{
    double sat = DMIN(threshMAX, (cass * cass) / k_rate);
    double sat2 = DMIN(threshMAX, (cass * cass) / k_rate2);
    double c = DMIN(cass, threshMAXCa);
    k->k12 = k12cf * sat2;
    k->k23 = k23cf * sat;
    k->k34 = k34cf * sat;
    k->k54 = k54cf * sat;
    k->k25 = k25cf * sat;
    k->k56 = k56cf * sat;
    k->regime = (c < threshCa56to8) ? 0 : ((c < threshCa34to7) ? 1 : 2);
}

/* RyR exit row; resolves the merged pseudo-states 7 (3/4) and 8 (5/6) by the
 * rules of the three Ca regimes (fru_rates_local.c:384-736).  May consume one
 * uniform and may rewrite *s. */
static void ryr_row(exit_row *e, int *s, const ryr_k *k, int *mti, uint32_t mt[MTN])
{
    double a1, a2, a3;
    switch (k->regime) {
    case 0: /* low Ca: the six real states, 7/8 resolved by a draw */
        if (*s == 7) *s = (orc_next(mti, mt) < (k->k34 / (k->k34 + k43))) ? 4 : 3;
        else if (*s == 8) *s = (orc_next(mti, mt) < k->k56 / (k->k56 + k65)) ? 6 : 5;
        switch (*s) {
        case 1: row2(e, k->k12, 2); break;
        case 2: row4(e, k21 + k->k23 + k->k25, k21, 1, k->k23, 3, k->k25, 5); break;
        case 3: row3(e, k32 + k->k34, k32, 2, k->k34, 4); break;
        case 4: row3(e, k43 + k45, k43, 3, k45, 5); break;
        case 5: row4(e, k52 + k->k54 + k->k56, k52, 2, k->k54, 4, k->k56, 6); break;
        case 6: row2(e, k65, 5); break;
        default: e->r[0] = 0.0; e->len = 1; break;
        }
        break;
    case 1: /* intermediate Ca: 5/6 merged into 8, 7 resolved by a draw */
        if (*s == 7) *s = (orc_next(mti, mt) < k->k34 / (k->k34 + k43)) ? 4 : 3;
        if (*s == 5 || *s == 6) *s = 8;
        switch (*s) {
        case 1: row2(e, k->k12, 2); break;
        case 2: row4(e, k21 + k->k23 + k->k25, k21, 1, k->k23, 3, k->k25, 8); break;
        case 3: row3(e, k32 + k->k34, k32, 2, k->k34, 4); break;
        case 4: row3(e, k43 + k45, k43, 3, k45, 8); break;
        case 8:
            a1 = k65 / (k->k56 + k65); a2 = a1 * k52; a3 = a1 * k->k54;
            row3(e, a2 + a3, a2, 2, a3, 4); break;
        default: e->r[0] = 0.0; e->len = 1; break;
        }
        break;
    default: /* high Ca: 3/4 merged into 7 and 5/6 into 8 */
        if (*s == 3 || *s == 4) *s = 7;
        else if (*s == 5 || *s == 6) *s = 8;
        switch (*s) {
        case 1: row2(e, k->k12, 2); break;
        case 2: row4(e, k21 + k->k23 + k->k25, k21, 1, k->k23, 7, k->k25, 8); break;
        case 7:
            a1 = k->k34 / (k43 + k->k34); a2 = (1.0 - a1) * k32; a3 = a1 * k45;
            row3(e, a2 + a3, a2, 2, a3, 8); break;
        case 8:
            a1 = k65 / (k->k56 + k65); a2 = a1 * k52; a3 = a1 * k->k54;
            row3(e, a2 + a3, a2, 2, a3, 7); break;
        default: e->r[0] = 0.0; e->len = 1; break;
        }
        break;
    }
}

/* All exit tables of one FRU and the largest total exit rate. */
typedef struct {
    exit_row lcc[NCLEFT];
    double vdi[NCLEFT];
    exit_row ryr[NCLEFT][NRYR];
    double cl[NCLEFT];
} fru_tables;

static double fru_tables_eval(fru_tables *T, int ltype[NCLEFT][2], int ryr[NCLEFT][NRYR], const int ito2[NCLEFT],
                              double V, const double frus[5], int *mti, uint32_t mt[MTN])
{
    int c, i;
    double alpha = alphacf * exp(0.012 * (V - 35.0));
    double beta = betacf * exp(-0.05 * (V - 35.0));
    /* voltage-dependent inactivation gate, :345-369 */
    double nu = 1;
    double yinf = nu * (0.4 / (1.0 + exp((V + 12.5) / 5.0)) + (1.0 - 0.4));
    double tau = 60.0 + 340.0 / (1.0 + exp((V + 30.0) / 12.0));
    double mx = 0.0;
    ryr_k k;
    for (c = 0; c < NCLEFT; c++) lcc_row(&T->lcc[c], ltype[c][0], alpha, beta, gammacf * frus[c + 1]);
    for (c = 0; c < NCLEFT; c++) T->vdi[c] = (ltype[c][1] == 2) ? (1.0 - yinf) / tau : yinf / tau;
    for (c = 0; c < NCLEFT; c++) {
        ryr_constants(&k, frus[c + 1]);
        for (i = 0; i < NRYR; i++) ryr_row(&T->ryr[c][i], &ryr[c][i], &k, mti, mt);
    }
    for (c = 0; c < NCLEFT; c++) T->cl[c] = (ito2[c] == 1) ? kfIto2 * frus[c + 1] : kbIto2;
    for (c = 0; c < NCLEFT; c++) {
        mx = DMAX(mx, T->lcc[c].r[0]);
        mx = DMAX(mx, T->vdi[c]);
        mx = DMAX(mx, T->cl[c]);
        for (i = 0; i < NRYR; i++) mx = DMAX(mx, T->ryr[c][i].r[0]);
    }
    return mx;
}

/* Same outputs as the reference's fru_rates_local (for pinning). */
double orc_fru_rates(int *ltype, int *ryr, int *ito2, const double dep[3], const double frus[5],
                     double *lrates, int *lindex, int *llen, double *vdep, double *rrates, int *rindex,
                     int *rlen, double *ito2rate, int *mti, uint32_t *mt)
{
    fru_tables T;
    int c, i, j;
    double mx = fru_tables_eval(&T, (int(*)[2])ltype, (int(*)[NRYR])ryr, ito2, dep[0], frus, mti, mt);
    for (c = 0; c < NCLEFT; c++) {
        for (j = 0; j < T.lcc[c].len; j++) {
            lrates[c * 4 + j] = T.lcc[c].r[j];
            if (j) lindex[c * 4 + j] = T.lcc[c].dest[j];
        }
        llen[c] = T.lcc[c].len;
        vdep[c] = T.vdi[c];
        ito2rate[c] = T.cl[c];
        for (i = 0; i < NRYR; i++) {
            for (j = 0; j < T.ryr[c][i].len; j++) {
                rrates[(c * NRYR + i) * 4 + j] = T.ryr[c][i].r[j];
                if (j) rindex[(c * NRYR + i) * 4 + j] = T.ryr[c][i].dest[j];
            }
            rlen[c * NRYR + i] = T.ryr[c][i].len;
        }
    }
    return mx;
}

/* ---- local Ca ODE: fcn_fru.c:23-137 --------------------------------------- */
void orc_fcn_fru(const double y[5], const double dep[3], const double lopen[NCLEFT], const int nopen[NCLEFT],
                 double dy[5])
{
    const double JDHconstant = 1.0 / (2.0 * VSS * Faraday * 1000.0);
    double V = dep[0], Cai = dep[1], CaNSR = dep[2], CaJSR = y[0];
    double JRyR[NCLEFT], Jxfer[NCLEFT], Jss[NCLEFT], JDH[NCLEFT], bSS[NCLEFT];
    double Jtr, JRyRtot, VFRT, VFsqRT, e2, a1, a2, bJSR;
    int c;
    Jtr = (CaNSR - CaJSR) / tautr;
    for (c = 0; c < NCLEFT; c++) JRyR[c] = JRyRmax * ((double)nopen[c]) * (CaJSR - y[c + 1]);
    JRyRtot = JRyR[0] + JRyR[1] + JRyR[2] + JRyR[3];
    for (c = 0; c < NCLEFT; c++) Jxfer[c] = (y[c + 1] - Cai) / tauxfer;
    for (c = 0; c < NCLEFT; c++) Jss[c] = (y[c + 1] - y[(c + 1) % NCLEFT + 1]) / tauss2ss;
    VFRT = V / RT_over_F;
    VFsqRT = (1000.0 * Faraday) * VFRT;
    e2 = exp(2.0 * VFRT);
    if (fabs(V) < 1.e-6) {
        for (c = 0; c < NCLEFT; c++)
            JDH[c] = -PCa * 2.0 * 1000.0 * Faraday * (y[c + 1] - Cao * 0.341) * lopen[c] * JDHconstant;
    } else {
        a2 = PCa * 4.0 * VFsqRT / (e2 - 1.0) * JDHconstant;
        for (c = 0; c < NCLEFT; c++) JDH[c] = -(y[c + 1] * e2 - Cao * 0.341) * a2 * lopen[c];
    }
    for (c = 0; c < NCLEFT; c++) {
        a1 = BSRtot * KBSR / ((y[c + 1] + KBSR) * (y[c + 1] + KBSR));
        a2 = BSLtot * KBSL / ((y[c + 1] + KBSL) * (y[c + 1] + KBSL));
        bSS[c] = 1.0 / (1.0 + a1 + a2);
    }
    a1 = CSQNtot * KmCSQN / ((CaJSR + KmCSQN) * (CaJSR + KmCSQN));
    bJSR = 1.0 / (1.0 + a1);
    dy[0] = bJSR * (Jtr - VSS / VJSR * JRyRtot);
    for (c = 0; c < NCLEFT; c++)
        dy[c + 1] = bSS[c] * (JDH[c] + JRyR[c] - Jxfer[c] - Jss[c] + Jss[(c + NCLEFT - 1) % NCLEFT]);
}

/* ---- one FRU over [t0,tf]: simfru_local.c:32-278 --------------------------- */
static int lcc_open(const int lt[2]) { return (lt[0] == 6 || lt[0] == 12) && lt[1] == 2; }
static int ryr_open(int s) { return s == 3 || s == 4 || s == 7; }

/* Categorical selection of simfru_local.c:217-226: leave the state when
 * u > 1 - dt*total, then walk the cumulative sum. */
static int pick(const exit_row *e, double dt, double u, int cur)
{
    double acc = 1.0 - dt * e->r[0];
    int n = 1;
    if (!(u > acc)) return cur;
    acc += dt * e->r[1];
    while (u > acc && n + 1 < e->len) {
        n++;
        acc += dt * e->r[n];
    }
    return e->dest[n];
}

/* FRU-substeps taken by orc_simfru since the library was loaded (the
 * workload unit; the CPU stand-in of the native API reports it). */
static unsigned long long orc_substeps_total = 0;
unsigned long long orc_substep_count(void) { return orc_substeps_total; }

void orc_simfru(double t0, double tf, const double dep0[3], const double depf[3], int ltype[NCLEFT][2],
                int ryr[NCLEFT][NRYR], int ito2[NCLEFT], double frus[5], int *mti, uint32_t mt[MTN])
{
    double span[3], dep[3], lopen[NCLEFT], y1[5], k1[5], dF[5], u[32];
    double t = t0, interval = tf - t0, mx, dt, cmax;
    int nopen[NCLEFT], c, i, j;
    fru_tables T;
    for (i = 0; i < 3; i++) { span[i] = depf[i] - dep0[i]; dep[i] = dep0[i]; }
    for (c = 0; c < NCLEFT; c++) {
        lopen[c] = lcc_open(ltype[c]) ? 1.0 : 0.0;
        nopen[c] = 0;
        for (i = 0; i < NRYR; i++) nopen[c] += ryr_open(ryr[c][i]);
    }
    while (t < tf) {
        orc_substeps_total++;
        mx = fru_tables_eval(&T, ltype, ryr, ito2, dep[0], frus, mti, mt);
        /* substep size, :135-146 */
        dt = DMIN(0.1 / mx, 10.001e-3);
        cmax = 0.e-3;
        for (c = 0; c < NCLEFT; c++) cmax = DMAX(cmax, frus[c + 1]);
        if (cmax > 1.5e-3) dt = DMIN(dt, 5.001e-3);
        dt = DMIN(dt, tf - t);
        /* Heun (trapezoid) step with the pre-transition open flags, :149-173 */
        orc_fcn_fru(frus, dep, lopen, nopen, dF);
        for (i = 0; i < 5; i++) { k1[i] = dt * dF[i]; y1[i] = frus[i] + k1[i]; }
        t = t + dt;
        for (i = 0; i < 3; i++) dep[i] = dep0[i] + (t - t0) / interval * span[i];
        orc_fcn_fru(y1, dep, lopen, nopen, dF);
        for (i = 0; i < 5; i++) frus[i] = frus[i] + (k1[i] + dt * dF[i]) / 2.0;
        /* 32 uniforms, index cleft*8 + {0 LCC, 1 VDI, 2..6 RyR, 7 ClCh}, :211-253 */
        for (j = 0; j < 32; j++) u[j] = orc_next(mti, mt);
        for (c = 0; c < NCLEFT; c++) {
            const double *uc = u + 8 * c;
            int moved = 0;
            ltype[c][0] = pick(&T.lcc[c], dt, uc[0], ltype[c][0]);
            if (uc[1] >= 1.0 - dt * T.vdi[c]) ltype[c][1] = 3 - ltype[c][1];
            for (i = 0; i < NRYR; i++) {
                int ns = pick(&T.ryr[c][i], dt, uc[2 + i], -1);
                if (ns >= 0) { ryr[c][i] = ns; moved = 1; }
            }
            if (uc[7] >= 1.0 - dt * T.cl[c]) ito2[c] = 3 - ito2[c];
            lopen[c] = lcc_open(ltype[c]) ? 1.0 : 0.0;
            if (moved) {
                nopen[c] = 0;
                for (i = 0; i < NRYR; i++) nopen[c] += ryr_open(ryr[c][i]);
            }
        }
    }
}

/* Batch over packed arrays: ltype[n][8], ryr[n][20], ito2[n][4], frus[n][5],
 * mti[n], mt[n][624]. */
void orc_simfru_batch(int n, double t0, double tf, const double dep0[3], const double depf[3], int *ltype,
                      int *ryr, int *ito2, double *frus, int *mti, uint32_t *mt)
{
    int f;
    for (f = 0; f < n; f++)
        orc_simfru(t0, tf, dep0, depf, (int(*)[2])(ltype + 8 * (size_t)f), (int(*)[NRYR])(ryr + 20 * (size_t)f),
                   ito2 + 4 * (size_t)f, frus + 5 * (size_t)f, &mti[f], mt + (size_t)MTN * f);
}

/* ---- reductions: calc_fru_flux_local.c:28-77, calc_fru_avg_local.c:27-105 -- */
void orc_flux_sums(int n, const int *ltype, const int *ito2, const double *frus, double num[5])
{
    double ica = 0.0, oca = 0, scss = 0.0, sjsr = 0.0;
    int nio = 0, f, c;
    for (f = 0; f < n; f++)
        for (c = 0; c < NCLEFT; c++) {
            if (lcc_open(ltype + 8 * f + 2 * c)) { ica = ica + frus[5 * f + c + 1]; oca = oca + 1; }
            if (ito2[4 * f + c] == 2) nio = nio + 1;
        }
    for (f = 0; f < n; f++) {
        sjsr += frus[5 * f];
        for (c = 0; c < NCLEFT; c++) scss += frus[5 * f + c + 1];
    }
    num[0] = scss; num[1] = sjsr; num[2] = ica; num[3] = oca; num[4] = nio;
}

void orc_avg_sums(int n, const int *ltype, const int *ryr, const int *ito2, const double *frus, double num[11])
{
    double cass = 0.0, cajsr = 0.0, totss = 0.0, totjsr = 0.0, jryr = 0.0, pryr = 0.0;
    double pnorm = 0.0, pnv = 0.0, plo = 0.0, pio = 0.0;
    int ready = 0, f, c, i, no;
    for (f = 0; f < n; f++) {
        double jsr = frus[5 * f];
        cajsr = cajsr + jsr;
        totjsr = totjsr + jsr * (1.0 + CSQNtot / (KmCSQN + jsr));
        for (c = 0; c < NCLEFT; c++) {
            double ss = frus[5 * f + c + 1];
            const int *lt = ltype + 8 * f + 2 * c;
            cass = cass + ss;
            totss = totss + ss * (1.0 + BSRtot / (KBSR + ss) + BSLtot / (KBSL + ss));
            no = 0;
            for (i = 0; i < NRYR; i++) {
                int s = ryr[20 * f + 5 * c + i];
                no += ryr_open(s);
                ready += (s == 1 || s == 2);
            }
            jryr = jryr + JRyRmax * ((double)no) * (jsr - ss);
            pryr = pryr + ((double)no);
            if (lt[0] <= 6) pnorm = pnorm + 1.0;
            if (lt[1] == 2) pnv = pnv + 1.0;
            if (lcc_open(lt)) plo = plo + 1.0;
            if (ito2[4 * f + c] == 2) pio = pio + 1.0;
        }
    }
    num[0] = cass; num[1] = cajsr; num[2] = jryr; num[3] = pryr; num[4] = (double)ready;
    num[5] = totss; num[6] = totjsr; num[7] = pnorm; num[8] = pnv; num[9] = plo; num[10] = pio;
}

/* Flux numerators -> (Jxfer, Jtr, ICa, Ito2), mpi_master.c:401-468 (and the
 * identical algebra of send_calc_fru_flux, :55-112).  dep = (V, Cai, CaNSR). */
void orc_currents(int nfru, double scale, const double dep[3], const double num[5], double out[4])
{
    double V = dep[0], Cai = dep[1], CaNSR = dep[2];
    double VFRT = V / RT_over_F, VFsqRT = (1000.0 * Faraday) * VFRT;
    double e1 = exp(VFRT), e2 = e1 * e1, icanum, ica, ito2, jtr, jxfer;
    if (fabs(V) < 1.e-6) {
        icanum = num[2] - num[3] * Cao * 0.341;
        ica = PCa * 2.0 * 1000.0 * Faraday * icanum;
        ica = ica / Acap;
        ito2 = ((double)num[4]) * PCl * 1000.0 * Faraday * (Clo - Cli);
        ito2 = ito2 / Acap;
    } else {
        icanum = num[2] * e2 - num[3] * Cao * 0.341;
        ica = PCa * 4.0 * VFsqRT * icanum / (e2 - 1.0);
        ica = ica / Acap;
        ito2 = ((double)num[4]) * PCl * VFsqRT * (Cli - Clo * e1) / (1.0 - e1);
        ito2 = ito2 / Acap;
    }
    jtr = (((double)nfru) * CaNSR - num[1]) / tautr;
    jxfer = (num[0] - ((double)nfru * (double)NCLEFT) * Cai) / tauxfer;
    out[0] = scale * jxfer;
    out[1] = scale * jtr;
    out[2] = scale * ica;
    out[3] = scale * ito2;
}
