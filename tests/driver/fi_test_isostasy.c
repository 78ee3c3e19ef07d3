/*
 * fi_test_isostasy.c — the reference driver's call sequence through the C
 * ABI of libfigpu.so (test infrastructure).
 *
 * Replays tests/test_isostasy.f90:337-402 of the reference for its disc
 * experiment test1d (par/test_isostasy_test1d.nml values, a 1000 km /
 * 1000 m ice disc switched on after t = 0):
 *
 *     bsl_init; isos_init; isos_init_state
 *     do n = 1, nt:  time = time_init + (n-1)*dtt
 *                    H_ice = interp_2d(time_ice, T_ice, time)
 *                    bsl_update(bsl, time); isos_update(isos, H_ice, time, bsl)
 *                    every dt_out: write isos%out
 *     isos_end
 *
 * Usage: fi_test_isostasy OUT_FILE PRECISION N DX NT DTT DT_OUT
 * Writes, for every output time, the record [time, z_bed(N*N), w(N*N),
 * we(N*N), maskocean(N*N) as 0/1 doubles] as raw doubles, x fastest.
 * Exit status: 0, or the FI_* status of the first failing call (after its
 * message on stderr), or 100 for a usage or I/O error.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fi_gpu.h"

static int check(fi_handle* h, int rc, const char* where)
{
    if (rc != FI_OK) {
        const char* m = h ? fi_last_error(h) : "";
        fprintf(stderr, "%s: status %d: %s\n", where, rc, m ? m : "");
    }
    return rc;
}

/* &isostasy of the disc experiment test1d, after isos_par_load's units */
static void test1d_params(fi_params* p, int precision)
{
    memset(p, 0, sizeof(*p));
    p->method = 3;
    p->lumping = 5;                 /* freqdomain */
    p->visc_scaling_method = 1;
    p->nl = 1;
    p->dt_method = 2;               /* tsit54 */
    p->precision = precision;
    p->dt_diagnostics = 10.0;
    p->viscosity_scaling = 1.0;
    p->zl[0] = 88.0e3;
    p->viscosities[0] = 1e21;
    p->eta_ref = 1e21;
    p->E = 66.0;
    p->nu = 0.28;
    p->rho_water = 1000.0;
    p->rho_ice = 910.0;
    p->rho_seawater = 1028.0;
    p->rho_uppermantle = 3400.0;
    p->g = 9.81;
    p->r_earth = 6.378e6;
    p->m_earth = 5.972e24;
    p->atol = 1e-2;
    p->rtol = 1e-4;
    p->dt_min = 1e-10;
    p->dt_max = 10.0;
    p->dt_init = 1.0;
    p->q = 1.0;
    p->tau = 3000.0;
}

int main(int argc, char** argv)
{
    if (argc != 8) {
        fprintf(stderr, "usage: %s OUT_FILE PRECISION N DX NT DTT DT_OUT\n", argv[0]);
        return 100;
    }
    const char* path = argv[1];
    const int precision = atoi(argv[2]), n = atoi(argv[3]), nt = atoi(argv[5]);
    const double dx = atof(argv[4]), dtt = atof(argv[6]), dt_out = atof(argv[7]);
    const double time_init = 0.0, r0 = 1000e3, h0 = 1000.0;
    const size_t cells = (size_t)n * n;
    FILE* fo = fopen(path, "wb");
    if (!fo || n < 4 || nt < 1) return 100;

    /* T_ice: no ice at time_ice(1) = time_init, the disc after it
     * (tests/test_isostasy.f90:222-239) */
    double* z_bed = (double*)calloc(cells, sizeof(double));
    double* H0 = (double*)calloc(cells, sizeof(double));
    double* H1 = (double*)calloc(cells, sizeof(double));
    double* H = (double*)calloc(cells, sizeof(double));
    double *o_zb = (double*)calloc(cells, sizeof(double)), *o_w = (double*)calloc(cells, sizeof(double));
    double* o_we = (double*)calloc(cells, sizeof(double));
    uint8_t* o_mo = (uint8_t*)calloc(cells, 1);
    double* rec = (double*)malloc(sizeof(double) * (1 + 4 * cells));
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            const double x = (i - (n - 1) / 2.0) * dx, y = (j - (n - 1) / 2.0) * dx;
            z_bed[(size_t)j * n + i] = 1e6;   /* bed far above sea level: no ocean */
            H1[(size_t)j * n + i] = (x * x + y * y <= r0 * r0) ? h0 : 0.0;
        }

    fi_params p;
    test1d_params(&p, precision);
    fi_bsl bsl;
    memset(&bsl, 0, sizeof(bsl));   /* bsl_init: method "const", bsl_init 0 */
    bsl.constant_ocean_surface = 1;
    bsl.A_ocean_pd = bsl.A_ocean_now = 3.625e14;
    int rc = check(NULL, fi_bsl_update(&bsl, time_init), "bsl_init");
    fi_handle* h = NULL;
    if (!rc) rc = check(h, fi_create(&p, n, n, dx, dx, NULL, &h), "isos_init");
    if (!rc) rc = check(h, fi_init_state(h, z_bed, H0, time_init, &bsl), "isos_init_state");

    fi_out out;
    memset(&out, 0, sizeof(out));
    out.z_bed = o_zb;
    out.w = o_w;
    out.we = o_we;
    out.maskocean = o_mo;
    for (int k = 1; k <= nt && !rc; ++k) {
        const double time = time_init + (k - 1) * dtt;
        const double* Hk = time > time_init ? H1 : H0;   /* interp_2d of the two slices */
        memcpy(H, Hk, cells * sizeof(double));
        if ((rc = check(h, fi_bsl_update(&bsl, time), "bsl_update"))) break;
        if ((rc = check(h, fi_update(h, H, time, &bsl, &out), "isos_update"))) break;
        if (fmod(time - time_init, dt_out) == 0.0) {
            rec[0] = time;
            memcpy(rec + 1, o_zb, cells * sizeof(double));
            memcpy(rec + 1 + cells, o_w, cells * sizeof(double));
            memcpy(rec + 1 + 2 * cells, o_we, cells * sizeof(double));
            for (size_t e = 0; e < cells; ++e) rec[1 + 3 * cells + e] = o_mo[e] ? 1.0 : 0.0;
            if (fwrite(rec, sizeof(double), 1 + 4 * cells, fo) != 1 + 4 * cells) rc = 100;
        }
    }
    if (h) {
        const int rd = fi_destroy(h);
        if (!rc) rc = check(NULL, rd, "isos_end");
    }
    fclose(fo);
    free(z_bed); free(H0); free(H1); free(H); free(o_zb); free(o_w); free(o_we); free(o_mo); free(rec);
    return rc;
}
