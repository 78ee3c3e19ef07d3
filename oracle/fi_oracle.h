/*
 * fi_oracle.h — CPU FP64 restatement of FastIsostasy's LV-ELVA hot path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only the test suite, the smoke
 * check and the CPU-baseline leg of the benchmark load this library, and
 * only as the checker (or as the timed CPU baseline).  The GPU library
 * never links it.
 *
 * Parity status: UNPINNED against reference outputs.  The reference is
 * Fortran + FFTW + NetCDF and none of those toolchains exist here, and the
 * reference stores no golden vectors.  This restatement is pinned instead
 * (a) to the transforms' mathematical definitions (DFT/DHT checked against
 * numpy and explicit cas matrices), (b) to the reference's only known
 * answer, the analytical ELVA disk of src/isostasy_benchmarks.f90:206-367,
 * and (c) to an independent numpy restatement of calc_lvelva.
 *
 * Array layout follows the reference: a field (nx, ny) is stored with x
 * fastest (Fortran column-major), i.e. element (i, j) at [j*nx + i] with
 * 0-based i, j.  All floating point is double (the reference built with
 * wp = dp, src/precision.f90:10), keeping the reference's single-precision
 * literal quirks where they change values.
 */
#ifndef FI_ORACLE_H
#define FI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters after isos_par_load's unit conversions
 * (src/fastisostasy.f90:925-1015): lengths in m, E in GPa. */
typedef struct {
    int32_t method;                 /* 0 none, 1 LLRA, 2 LV-ELRA, 3 LV-ELVA */
    int32_t interactive_sealevel;
    int32_t include_elastic;
    int32_t heterogeneous_ssh;
    int32_t correct_compression;
    int32_t lithosphere;            /* 0 uniform, 1 gaussian_plus, 2 gaussian_minus, 3 caller field */
    int32_t mantle;                 /* 0 uniform, 1 gaussian_plus, 2 gaussian_minus, 3 caller field */
    int32_t layering;               /* 0 equalized, 1 parallel */
    int32_t lumping;                /* 0 bottom, 1 min, 2 max, 3 mean, 4 logmean, 5 freqdomain */
    int32_t visc_scaling_method;    /* 0 none, 1 scale, 2 min, 3 max */
    int32_t nl;
    int32_t dt_method;              /* 0 euler, 1 rk4, 2 tsit54 */
    int32_t stage_mode;             /* 0 reference-compatible, 1 true stages */
    int32_t nx_target, ny_target;   /* 0: reference padding rule */
    int32_t pad_;
    double dt_diagnostics, min_pad, viscosity_scaling;
    double zl[8], viscosities[8], dl, eta_ref;
    double E, nu, rho_water, rho_ice, rho_seawater, rho_uppermantle, rho_litho, g;
    double r_earth, m_earth;
    double atol, rtol, dt_min, dt_max, dt_init, q;
    double tau;                     /* [yr] asthenosphere relaxation time (methods 0-2) */
} orc_params;

typedef struct {
    int32_t method;                 /* 0 const, 1 file, 2 fastiso, 3 mixed */
    int32_t constant_ocean_surface;
    int32_t n_series, n_aocean;
    double bsl_init, bsl_now, A_ocean_now, A_ocean_pd, time;
    const double *series_t, *series_v;   /* method file/mixed */
    const double *bsl_vec, *aocean_vec;  /* A_ocean(bsl) table */
} orc_bsl;

typedef struct orc_model orc_model;

/* --- transforms ------------------------------------------------------- */
void orc_cfft(int n, double *re, double *im, int sign);            /* in place, unnormalised */
void orc_dht2d(int nx, int ny, const double *in, double *out);      /* FFTW_DHT x FFTW_DHT */
void orc_rfft2_conv(int nx, int ny, int M, const double *kspec_re, const double *kspec_im,
                    const double *in, double *out);
void orc_kernel_spectrum(int nx, int ny, int M, const double *kernel, double *spec_re, double *spec_im);

/* --- pieces of the path ------------------------------------------------ */
void orc_derivative_x(double *d, const double *u, const double *dx, int nx, int ny);
void orc_derivative_y(double *d, const double *u, const double *dy, int nx, int ny);
void orc_derivative_xx(double *d, const double *u, const double *dx, int nx, int ny);
void orc_derivative_yy(double *d, const double *u, const double *dy, int nx, int ny);
void orc_kappa(double *kappa, int nx, int ny, double dx, double dy);
void orc_lvelva(double *dwdt, const double *w, const double *canom_full, const uint8_t *mask,
                double g, double nu, const double *D, const double *eta, const double *R,
                const double *kappa, int nx, int ny, const double *dxm, const double *dym,
                double sec_per_year);
void orc_elastic_green(double *filt, int nx, int ny, double dx, double dy);
void orc_zss_green(double *filt, int nx, int ny, double m_earth, double r_earth, double dx, double dy);
void orc_conv(double *out, int nx, int ny, int M, const double *spec_re, const double *spec_im,
              const double *in);

/* --- whole model ------------------------------------------------------- */
orc_model *orc_create(const orc_params *p, int nx_ice, int ny_ice, double dx, double dy,
                      const double *K_or_null);
void orc_destroy(orc_model *m);
int  orc_dims(const orc_model *m, int32_t *out8);   /* nx ny icrop1 icrop2 jcrop1 jcrop2 nx_ice ny_ice */
int  orc_set_fields(orc_model *m, const double *D, const double *eta_eff, const double *R,
                    const uint8_t *maskactive);
int  orc_init_ref(orc_model *m, const double *z_bed, const double *H_ice, double bsl,
                  const double *dz_ss_or_null);
int  orc_init_state(orc_model *m, const double *z_bed, const double *H_ice, double time,
                    orc_bsl *bsl);
int  orc_update(orc_model *m, const double *H_ice, double time, orc_bsl *bsl);
void orc_bsl_update(orc_bsl *bsl, double year_bp);
int  orc_get_field(const orc_model *m, int which, double *out);   /* padded grid */
int  orc_get_scalars(const orc_model *m, double *out16);
void orc_rhs_now(orc_model *m, double *dwdt);   /* get_dwdt at the current state */
void orc_set_threads(int n);
void orc_set_reuse_frozen(int on);          /* bit-identical reuse of the frozen RHS */
void orc_set_max_rejections(long n);        /* per isos_update; 0 = default 1e6 */
void orc_set_smooth_convolution(int on);    /* 2/3/5/7-smooth convolution size (timed baselines) */
void orc_set_rhs_noise(double eps, unsigned long long seed);   /* conditioning probe, tests only */

/* The Kelvin-function table of LV-ELRA (1001 entries each). */
void orc_kei_table(double *rn, double *kei);

/* rheology_file branch helpers (src/fastisostasy.f90:262-420) */
void orc_bilinear_array(const double *x, int nxr, const double *y, int nyr, const double *z,
                        const double *xo, int nx, const double *yo, int ny, double *out);
double orc_interp_0d(const double *x, const double *y, int n, double xout);
int orc_smooth_gauss_2d(double *var, int nx, int ny, double dx, double sigma);
void orc_lump3(const double *eta3, const double *bnd, const double *kappa, int n, int nl, int lumping,
               double *eta_eff, double *R);

#ifdef __cplusplus
}
#endif
#endif
