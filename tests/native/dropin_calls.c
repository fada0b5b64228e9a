/*
 * Test program for the drop-in layer: calls the reference's MPI-layer entry
 * points (parameters.h:255-271) in the order caf.c and rk_pd54m.c make them
 * -- initialize_mpi, initialize_mpi_state, send_calc_fru_flux, then stages
 * of distrib_simFRU between send_save_state / send_resume_state, then
 * send_calc_fru_avg, parallel_get_FRUs and end_mpi -- and prints every result.
 * Linked once against libgw_fru.so (FRUs on the GPU) and once against the
 * CPU stand-in over the oracle; the two outputs are compared by the tests.
 * Lines: "J <4 currents>", "O <12 otherstates>", "I <integer checksums>",
 * "F <sums of the FRU Ca states>".
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "gw_fru.h"

#define N 96
int NFRU_sim = N;                      /* caf.c:34-36, read by the library */
double NFRU_scale = 12500.0 / N;

static double frus[N][5];
static int ltype[N][4][2], ryr[N][4][5], ito2[N][4], mti[N];
static unsigned long mt[N][625];

static void knuth_seed(unsigned long *m, uint32_t seed)
{
    uint32_t x = seed;
    m[0] = x;
    for (uint32_t i = 1; i < 624; i++) {
        x = 1812433253u * (x ^ (x >> 30)) + i;
        m[i] = x;
    }
}

static void print_j(double a, double b, double c, double d) { printf("J %.17g %.17g %.17g %.17g\n", a, b, c, d); }

int main(int argc, char **argv)
{
    int rank = -1, procs = -1, f, c, k;
    double J[4], dep0[3] = {-94.7, 8.0e-5, 0.26}, depf[3], state[37] = {0}, other[12];
    for (f = 0; f < N; f++) {  /* a varied start: every LCC / RyR state class */
        frus[f][0] = 0.3 + 0.005 * f;
        for (c = 0; c < 4; c++) {
            frus[f][c + 1] = 1.0e-4 * (1 + (f + c) % 7);
            ltype[f][c][0] = 1 + (f + 3 * c) % 12;
            ltype[f][c][1] = 1 + (f + c) % 2;
            for (k = 0; k < 5; k++) ryr[f][c][k] = 1 + (f + c + k) % 8;
            ito2[f][c] = 1 + (f * c) % 2;
        }
        knuth_seed(mt[f], 5489u + (uint32_t)f);
        mti[f] = (f * 37) % 625;
    }
    initialize_mpi(&argc, argv, &rank, &procs);
    printf("I %d %d\n", rank, procs);
    initialize_mpi_state(frus, ltype, ryr, ito2, mti, mt);
    send_calc_fru_flux(dep0, &J[0], &J[1], &J[2], &J[3]);
    print_j(J[0], J[1], J[2], J[3]);
    double t = 10.0;
    for (k = 0; k < 12; k++) {
        const double dt = 0.004 * (1 + k % 3);
        depf[0] = dep0[0] + 9.0 * (k + 1);  /* an upstroke: -94.7 -> +13 mV */
        depf[1] = dep0[1] * 1.01;
        depf[2] = dep0[2];
        send_save_state();
        distrib_simFRU(t, t + dt, dep0, depf, &J[0], &J[1], &J[2], &J[3]);
        print_j(J[0], J[1], J[2], J[3]);
        if (k % 3 == 2) {  /* a rejected attempt, retried with half the step */
            send_resume_state();
            distrib_simFRU(t, t + dt / 2, dep0, depf, &J[0], &J[1], &J[2], &J[3]);
            print_j(J[0], J[1], J[2], J[3]);
            t += dt / 2;
        } else {
            t += dt;
        }
        dep0[0] = depf[0];
        dep0[1] = depf[1];
    }
    state[0] = dep0[0];
    state[6] = dep0[1];
    state[7] = dep0[2];
    send_calc_fru_avg(state, other);
    printf("O");
    for (k = 0; k < 12; k++) printf(" %.17g", other[k]);
    printf("\n");
    parallel_get_FRUs(frus, ltype, ryr, ito2, mt, mti);
    long long si = 0;
    unsigned long long x = 0;
    double sf[5] = {0};
    for (f = 0; f < N; f++) {
        for (c = 0; c < 4; c++) {
            si += ltype[f][c][0] * 3 + ltype[f][c][1] * 5 + ito2[f][c] * 7;
            for (k = 0; k < 5; k++) si += ryr[f][c][k] * (k + 11);
        }
        si += mti[f];
        for (k = 0; k < 624; k++) x = x * 1099511628211ull ^ mt[f][k];
        for (k = 0; k < 5; k++) sf[k] += frus[f][k];
    }
    printf("I %lld %llu\n", si, x);
    printf("F %.17g %.17g %.17g %.17g %.17g\n", sf[0], sf[1], sf[2], sf[3], sf[4]);
    end_mpi();
    return 0;
}
