/*
 * fi_gpu.h — C ABI of the GB300 LV-ELVA library (libfigpu.so).
 *
 * Drop-in boundary for FastIsostasy's time stepping: LV-ELVA (method 3),
 * and LLRA / LV-ELRA (methods 0-2) on the same update path.  Each entry
 * point replaces one reference routine of module `fastisostasy`
 * (src/fastisostasy.f90) or `barysealevel` (src/barysealevel.f90); the
 * Fortran caller keeps its isos_class / bsl_class and binds these functions
 * through iso_c_binding (module fastisostasy_gpu, fastisostasy_gpu.f90).
 *
 * Conventions
 *   - Arrays are plain host pointers in the reference's Fortran layout:
 *     a field (nx, ny) is contiguous with x fastest.  "Ice grid" arrays are
 *     (nx_ice, ny_ice); "padded" arrays are (nx, ny) of the padded domain
 *     (fi_dims).  Masks are uint8_t 0/1 (Fortran logical on the caller side
 *     converts with merge(1_c_int8_t, 0_c_int8_t, mask)).
 *   - Every call returns an int status; the reference `stop`s instead
 *     (e.g. src/fastisostasy.f90:197, 853, 868, 897).  fi_last_error() gives
 *     the message.
 *   - Device buffers are owned by the handle; the caller owns every host
 *     array.  Each handle has its own CUDA stream; handles are independent
 *     and may be driven from different host threads.
 *   - There is no CPU fallback: fi_create fails with FI_E_CUDA when no CUDA
 *     device is usable.
 */
#ifndef FI_GPU_H
#define FI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FI_OK = 0,
    FI_E_NAN = 1,      /* NaN in z_bed (src/fastisostasy.f90:864-869) */
    FI_E_LARGE = 2,    /* |w|,|we| > 1e5 or |dz_ss| > 1e3 (check_isos_instabilities :874-899) */
    FI_E_STEP = 3,     /* adaptive step below dt_min or rejected too often (fi_set_max_rejections) */
    FI_E_OOM = 4,      /* device allocation failed */
    FI_E_CONFIG = 5,   /* unsupported configuration (the reference's `stop`s in isos_init) */
    FI_E_CUDA = 6,     /* CUDA runtime error */
    FI_E_TIMEOUT = 7,  /* a bounded device wait expired */
    FI_E_ARG = 8,      /* invalid argument */
    FI_E_STATE = 9,    /* call out of order (e.g. update before init_state) */
    FI_E_SIZE = 10,    /* grid larger than fi_lvelva_static's scratch (or odd-sized) */
    FI_E_CANCELLED = 11  /* solve request cancelled (fi_serve_cancel) */
};

enum { FI_PREC_FP64 = 0, FI_PREC_MIXED = 1 };

/* isos_param_class (src/isostasy_defs.f90:34-100) after isos_par_load's
 * unit conversion (src/fastisostasy.f90:925-1015): lengths in m, E in GPa.
 * String options are integer codes. */
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
    int32_t nl;                     /* viscous layers, 1..8 */
    int32_t dt_method;              /* 0 euler, 1 rk4, 2 tsit54 */
    int32_t stage_mode;             /* 0 reference-compatible stages, 1 true stages */
    int32_t nx_target, ny_target;   /* 0: reference square padding; else explicit even sizes */
    int32_t precision;              /* FI_PREC_FP64 or FI_PREC_MIXED */
    double dt_diagnostics, min_pad, viscosity_scaling;
    double zl[8], viscosities[8], dl, eta_ref;
    double E, nu, rho_water, rho_ice, rho_seawater, rho_uppermantle, rho_litho, g;
    double r_earth, m_earth;
    double atol, rtol, dt_min, dt_max, dt_init, q;
    double tau;                     /* [yr] asthenosphere relaxation time (methods 0-2) */
} fi_params;

/* bsl_class (src/barysealevel.f90:16-29); series arrays are caller-owned
 * tables replacing the reference's file readers. */
typedef struct {
    int32_t method;                 /* 0 const, 1 file, 2 fastiso, 3 mixed */
    int32_t constant_ocean_surface;
    int32_t n_series, n_aocean;
    double bsl_init, bsl_now, A_ocean_now, A_ocean_pd, time;
    const double *series_t, *series_v;
    const double *bsl_vec, *aocean_vec;
} fi_bsl;

/* isos_out_class (src/isostasy_defs.f90:185-200): ice-grid outputs, any
 * pointer may be NULL. */
typedef struct {
    double *z_bed, *z_ss, *dz_ss, *w, *we, *dwdt, *canom_full, *Hice;
    uint8_t *maskocean, *maskgrounded, *maskcontinent;
} fi_out;

typedef struct fi_handle fi_handle;

/* Replaces isos_init (src/fastisostasy.f90:64-473), method-3 branch:
 * domain padding (init_domain_size, src/isos_utils.f90:285-354), kappa,
 * rigidity, effective viscosity and R, Green's-function spectra, maskactive.
 * K_or_null is the padded (nx, ny) distortion field or NULL (K = 1). */
int fi_create(const fi_params* p, int nx_ice, int ny_ice, double dx, double dy, const double* K_or_null,
              fi_handle** out);
/* init_domain_size (src/isos_utils.f90:285-354) without creating anything:
 * nx, ny, icrop1, icrop2, jcrop1, jcrop2 of the padded domain fi_create
 * would build.  Callers size padded fields (fi_set_fields, fi_request) with it. */
int fi_padded_dims(const fi_params* p, int nx_ice, int ny_ice, double dx, double dy, int32_t* out6);
/* Replaces isos_end (src/fastisostasy.f90:911-923). */
int fi_destroy(fi_handle* h);
/* nx, ny, icrop1, icrop2, jcrop1, jcrop2 (1-based like the reference), nx_ice, ny_ice */
int fi_dims(const fi_handle* h, int32_t* out8);
/* Caller-computed padded fields (the rheology_file / mask_file branches of
 * isos_init, src/fastisostasy.f90:185-214, 262-417).  eta_eff is final.
 * Any pointer may be NULL (kept). */
int fi_set_fields(fi_handle* h, const double* D_lith, const double* eta_eff, const double* R,
                  const uint8_t* maskactive);
/* The rheology_file branches of isos_init (lithosphere and/or mantle =
 * "rheology_file", src/fastisostasy.f90:262-290, 340-420), from the arrays
 * its NetCDF reader returns (coordinates and fields as nc_read_and_scale_*
 * leaves them; fields x fastest, then y, then z).  On the device:
 * bilinear_interpolation onto the padded grid (single precision, flat
 * beyond the file's grid; src/isos_utils.f90:495-575), smooth_gauss_2D when
 * rheo_smoothing_radius > 0 (src/isos_utils.f90:696-819), the rigidity; per
 * file level the interpolated log10 viscosity (+ viscosity_scaling x its
 * stddev when stddev_scaling), clamped to [16, 23], interpolated in depth to
 * the layer boundaries (interp_0d), 10**, lumped (freqdomain R), smoothed;
 * then the viscosity scaling, compressibility and eta_ref transform.
 * Replaces the handle's lithosphere thickness and D_lith (thickness given)
 * and eta_eff and R (viscosity given).  Method 3 only.  FI_E_ARG for a
 * smoothing window wider than the grid (the reference stops there). */
typedef struct {
    int32_t nx, ny, nz;                   /* file grid */
    const double *xc, *yc, *zc;           /* ascending */
    const double* litho_thickness;        /* nx*ny, or NULL */
    double litho_thickness_scaling;
    const double* log10_viscosity;        /* nx*ny*nz, or NULL */
    const double* stddev_log10_viscosity; /* nx*ny*nz, or NULL */
    int32_t stddev_scaling;               /* viscosity_scaling_method = "stddev" */
    double rheo_smoothing_radius;         /* [m]; 0: none */
} fi_rheology;
int fi_set_rheology(fi_handle* h, const fi_rheology* r);
/* Replace the elastic (GE) and geoid (GN) Green's functions (padded (nx, ny),
 * centred like calc_elastic_green, src/green_functions.f90:43-91);
 * spectra are recomputed.  Either may be NULL. */
int fi_set_kernels(fi_handle* h, const double* GE, const double* GN);
/* Replaces isos_init_ref (src/fastisostasy.f90:550-575). */
int fi_init_ref(fi_handle* h, const double* z_bed, const double* H_ice, double bsl, const double* dz_ss_or_null);
/* Replaces isos_init_state (src/fastisostasy.f90:596-660), without restart. */
int fi_init_state(fi_handle* h, const double* z_bed, const double* H_ice, double time, fi_bsl* bsl);
/* Replaces isos_update (src/fastisostasy.f90:731-872).  H_ice is ice grid;
 * outputs are copied to `out` (may be NULL; so may each of its arrays).
 * Synchronous.  On ice grids of 65536 cells and more, arrays in page-locked
 * host memory (cudaHostAlloc, or ranges registered with cudaHostRegister)
 * are copied to and from the device directly; pageable arrays go through a
 * page-locked staging buffer of the handle. */
int fi_update(fi_handle* h, const double* H_ice, double time, fi_bsl* bsl, fi_out* out);
/* Asynchronous isos_update for device-resident inputs: d_H_ice is a DEVICE
 * pointer to the ice-grid thickness (NULL keeps the previous one).  Valid for
 * bsl methods const and file; returns before the work completes.  The read of
 * d_H_ice is ordered on the handle's stream (fi_stream / fi_set_stream): work
 * that fills it on another stream, including a plain cudaMemcpy from pageable
 * memory, must have completed or be ordered before that stream. */
int fi_update_async(fi_handle* h, const double* d_H_ice, double time, fi_bsl* bsl);
/* Waits for the handle's stream; returns the device status (FI_E_NAN, ...). */
int fi_synchronize(fi_handle* h);
/* Run metrics of a handle (no reference counterpart; the reference has no
 * instrumentation beyond gprof): one JSON object, NUL-terminated, in buf —
 * grid, form, integrator, updates made, model time and step, accepted and
 * rejected steps, adaptive attempts (tsit54), kernels enqueued, CUDA graphs
 * captured, host time inside the update calls, device status.  Waits for
 * the handle's stream.  FI_E_SIZE when len is too small (1 KiB suffices).
 * With the environment variable FI_METRICS_FILE set, fi_destroy appends
 * this line to that file (a per-run metrics sink).  The host API calls
 * also open NVTX ranges (fi_create, fi_update, ...) for timeline tools. */
int fi_metrics_json(fi_handle* h, char* buf, size_t len);
/* Step-control safety of the adaptive method (tsit54).  The reference
 * halves dt after a rejection without any floor (src/integrators.f90:196-198)
 * and reads dt_min (src/fastisostasy.f90:1008) without using it.  Here an
 * update fails with FI_E_STEP when a rejection would take dt below
 * fi_params.dt_min, or when more than max_per_update attempts are rejected
 * within one update (default 1e6; 0 restores it). */
int fi_set_max_rejections(fi_handle* h, int64_t max_per_update);
/* Replaces bsl_update (src/barysealevel.f90:195-252). */
int fi_bsl_update(fi_bsl* b, double year_bp);

/* Asynchronous output (no reference counterpart; the step loop's write of
 * isos%out every dt_out, src/isostasy_io.f90:56-465, without a stall):
 * fi_output_async snapshots the isos%out fields on the device in stream
 * order, after the updates enqueued so far, and copies them to dst on a
 * side stream while later updates run.  dst holds fi_output_bytes(h) bytes
 * (page-locked memory lets the copy overlap): 11 ice-grid fields of doubles,
 * x fastest, in the order z_bed, z_ss, dz_ss, w, we, dwdt, canom_full,
 * Hice, maskocean, maskgrounded, maskcontinent (masks as 0.0 / 1.0).  One
 * snapshot is staged at a time: the next fi_output_async orders itself
 * after the previous copy on the device.  fi_output_wait returns when the
 * last copy has landed. */
int64_t fi_output_bytes(const fi_handle* h);
int fi_output_async(fi_handle* h, double* dst);
int fi_output_wait(fi_handle* h);

/* Inspection of padded fields; `which` follows FI_FIELD_*. */
enum {
    FI_FIELD_Z_BED = 0, FI_FIELD_DWDT = 1, FI_FIELD_W = 2, FI_FIELD_WE = 3, FI_FIELD_HAF = 4,
    FI_FIELD_HICE = 5, FI_FIELD_Z_SS = 6, FI_FIELD_DZ_SS = 7, FI_FIELD_CANOM_LOAD = 8,
    FI_FIELD_CANOM_FULL = 9, FI_FIELD_MASS_ANOM = 10, FI_FIELD_MASKOCEAN = 11, FI_FIELD_MASKGROUNDED = 12,
    FI_FIELD_MASKCONTINENT = 13, FI_FIELD_CANOM_MANTLE = 14, FI_FIELD_CANOM_LITHO = 15,
    FI_FIELD_CANOM_SEAWATER = 16, FI_FIELD_CANOM_ICE = 17, FI_FIELD_X = 18, FI_FIELD_KAPPA = 19,
    FI_FIELD_D_LITH = 20, FI_FIELD_ETA_EFF = 21, FI_FIELD_R = 22, FI_FIELD_MASKACTIVE = 23,
    FI_FIELD_GE = 24, FI_FIELD_GN = 25
};
int fi_get_field(fi_handle* h, int which, double* out_padded);
/* t, dt, time_diagnostics, bsl, V_af, V_den, deltaV_bsl, dbsl_total, n_rhs,
 * n_accept, n_reject, sec_per_year, compressibility, Vden_factor, conv size, bsl_ref */
int fi_get_scalars(fi_handle* h, double* out16);

/* calc_lvelva (src/lv_elva.f90:31-126) on padded host arrays with this
 * handle's rigidity, viscosity, kappa, R, maskactive and spacing. */
int fi_lvelva(fi_handle* h, const double* w, const double* canom_full, double* dwdt);
/* precomputed_fftconvolution (src/convolutions.f90:59-91) with the elastic
 * (kernel 0) or geoid (kernel 1) spectrum. */
int fi_convolve(fi_handle* h, int kernel, const double* in_padded, double* out_padded);

/* fi_lvelva_static has no counterpart in the reference: calc_lvelva
 * (src/lv_elva.f90:31-126) for callers that may not allocate device memory
 * once running (a coupled model that splits HBM among its components at
 * start-up; a loop that cannot afford cudaFree's device-wide sync).  All
 * arrays are DEVICE pointers of the caller, (nx, ny) with x fastest, double
 * except the 0/1 mask; d_kappa and d_R are the cell-layout fields of
 * calc_kappa / the viscous response (FI_FIELD_KAPPA, FI_FIELD_R).  Spacing
 * is uniform (dx, dy) when d_dx_matrix and d_dy_matrix are both NULL, else
 * they are the per-cell dx*K and dy*K of a distorted grid (both or neither).
 * The FP64 work is queued on `stream` (a cudaStream_t, NULL = legacy default
 * stream) and the call returns without waiting.  No device memory is
 * allocated: the scratch is one static device array sized for
 * nx, ny <= FI_STATIC_MAX_N (even, >= 4); other sizes return FI_E_SIZE.
 * The first call on a device (which must be current) loads the library's
 * device code; make it before capturing any stream.  Calls that can overlap
 * on one device race on the shared scratch and must be serialised by the
 * caller. */
#define FI_STATIC_MAX_N 256
int fi_lvelva_static(const double* d_w, const double* d_canom_full, const uint8_t* d_maskactive,
                     const double* d_D_lith, const double* d_eta_eff, const double* d_kappa, const double* d_R,
                     const double* d_dx_matrix, const double* d_dy_matrix, int nx, int ny, double dx, double dy,
                     double g, double nu, double sec_per_year, double* d_dwdt, void* stream);

/* ---- Solve server: continuous batching of independent solves ----------
 * No counterpart in the reference (a caller there runs one isos_class at a
 * time).  A request is one solve: fi_create + fi_set_fields + fi_init_state,
 * then isos_update every dtt from t0 to t_end with a constant ice load and
 * barystatic sea level.  One scheduler thread admits queued requests while
 * the in-flight cap and free device memory (less reserve_gb) allow, keeps
 * every running request's updates queued on its own stream so that requests
 * of different sizes overlap on the GPU, and retires finished requests
 * (their handles are freed).  A result does not depend on the mix it ran in.
 * An ensemble is a set of requests submitted together. */
typedef struct fi_server fi_server;
typedef struct {
    fi_params p;
    int32_t nx_ice, ny_ice;
    double dx, dy;
    const double* z_bed;          /* ice grid */
    const double* H_ref;          /* ice grid at t0 (the reference state), NULL = no ice */
    const double* H_ice;          /* ice grid, the load over the solve */
    const double* D_lith;         /* padded (fi_padded_dims) or NULL */
    const double* eta_eff;        /* padded or NULL */
    const double* R;              /* padded or NULL */
    const uint8_t* maskactive;    /* padded or NULL */
    double t0, t_end, dtt;        /* years */
    double bsl;                   /* barystatic sea level [m] */
} fi_request;
typedef struct {
    int32_t state;                /* 0 queued, 1 running, 2 done, 3 failed, 4 cancelled */
    int32_t status;               /* FI_* status of the solve */
    int64_t updates;              /* isos_update calls issued */
    double t_submit, t_admit, t_done;   /* seconds on the server clock */
    char error[128];              /* message of a failed solve */
} fi_request_info;
/* The server drives the device that is current when it is created.  A
 * request whose estimated device footprint plus reserve_gb exceeds the
 * device's memory is never admitted: it fails at once with FI_E_OOM.  One
 * that fits is admitted when free memory (less the reserve) allows, or when
 * nothing else runs; a device allocation that fails then fails it with
 * FI_E_OOM, and the server goes on with the others. */
int fi_serve_create(int max_inflight, double reserve_gb, fi_server** out);
/* Copies the request's arrays; returns at once. */
int fi_serve_submit(fi_server* s, const fi_request* r, uint64_t* id);
int fi_serve_info(fi_server* s, uint64_t id, fi_request_info* info);
/* Waits up to timeout_s for the request to finish (FI_E_TIMEOUT otherwise). */
int fi_serve_wait(fi_server* s, uint64_t id, double timeout_s, fi_request_info* info);
/* w and z_bed on the ice grid of a finished request (either may be NULL);
 * releases the request's record. */
int fi_serve_result(fi_server* s, uint64_t id, double* w_ice, double* z_bed_ice);
double fi_serve_clock(fi_server* s);
/* Cancels a request: a queued one at once; a running one stops issuing
 * updates and is retired (its handle freed) once those in flight finish,
 * without disturbing the other requests.  Its state becomes 4 and
 * fi_serve_result returns FI_E_CANCELLED.  FI_E_STATE if it already ended. */
int fi_serve_cancel(fi_server* s, uint64_t id);
/* Finishes every submitted request, then stops the scheduler. */
int fi_serve_destroy(fi_server* s);

/* Batched ensembles of handles driven in lockstep: one isos_update to `time`
 * for each of n handles (bsl[i] is handle i's bsl_class), each enqueued on
 * its handle's own stream without waiting, so members of different sizes
 * overlap on the device.  The ice load of each member is the one it already
 * holds.  fi_batch_synchronize waits for all and returns the first failing
 * status (per-member statuses in `status` if not NULL). */
int fi_batch_update(fi_handle* const* hs, int n, double time, fi_bsl* bsl);
int fi_batch_synchronize(fi_handle* const* hs, int n, int32_t* status);

/* Batched ensembles in shared launches: every member runs reference-
 * compatible tsit54 (stage_mode 0) in the same precision, initialised to the
 * same time.  fi_batch_step enqueues one isos_update to `time` for all
 * members as a single CUDA graph: the members' update heads as parallel
 * branches, then the adaptive Tsit5 attempts of all members in one loop of
 * batched launches (each launch covers every member that still has an
 * attempt left; accept/reject and step sizes stay per member), then the
 * update tails.  Each member's result is bit-identical to driving it alone
 * in FP64; in the mixed form the batched kernels may contract FP32
 * multiply-adds differently, so results agree to that rounding.  The
 * members' load is the one they hold.  Do not drive members on their own
 * while a batch step is in flight (fi_batch_wait first). */
typedef struct fi_batch fi_batch;
int fi_batch_create(fi_handle* const* hs, int n, fi_batch** out);   /* 1 <= n <= 2048 */
/* Scheduling priority of a batch's launches (no reference counterpart):
 * level 0 normal, 1 high (the device's greatest stream priority).  Several
 * batches stepping together (an ensemble split into groups) let the group
 * with the longest chain of attempts go first while the others fill the
 * SMs it leaves idle.  Only before the batch's first fi_batch_step. */
int fi_batch_set_priority(fi_batch* b, int level);
/* Autotuner of the batched passes (no reference counterpart): times the
 * first RHS of an attempt over all members on the device for candidate
 * shapes — stencil rows per column-strip task (8/16/32), rows per row-
 * transform block (2/4/8/16), spectrum columns per column-transform block
 * (1/2/4/8/16), resident-grid waves (2/4/8/16) — by coordinate descent,
 * and keeps the fastest.  Overwrites the members' RHS scratch (dead between
 * updates).  Only before the batch's first fi_batch_step.  chosen4 (or
 * NULL): rows, columns, strip rows, waves. */
int fi_batch_autotune(fi_batch* b, int32_t* chosen4);
int fi_batch_step(fi_batch* b, double time, fi_bsl* bsl);
int fi_batch_wait(fi_batch* b, int32_t* status);
int fi_batch_destroy(fi_batch* b);

/* The analytical ELVA disc (Bueler et al. 2007, eq. 17) as the reference's
 * disc benchmark writes it (isosbench_elva_disk,
 * src/isostasy_benchmarks.f90:74-280), evaluated on the device: a fast
 * validator for runs of the disc experiments.  out is (nx, ny) on the host. */
int fi_elva_disk(int nx, int ny, double dx, double r0, double h0, double eta, double D, double rho_ice,
                 double rho_m, double g, double time_yr, double* out);

/* Restart support: the complete device state (fields + integrator clock) as
 * doubles; bit-identical round trip. */
size_t fi_state_size(const fi_handle* h);
int fi_state_export(fi_handle* h, double* buf);
int fi_state_import(fi_handle* h, const double* buf);

/* The handle's CUDA stream (cudaStream_t) for event timing by the caller. */
void* fi_stream(fi_handle* h);
/* Run the handle's work on the caller's stream (cudaStream_t; NULL returns
 * to the handle's own), after the work already enqueued has finished.  The
 * caller keeps the stream alive while the handle uses it.  (The reference
 * has no streams; its FFTW plans are the handle's own state likewise.) */
int fi_set_stream(fi_handle* h, void* stream);
/* Number of kernels this handle has enqueued so far. */
long long fi_launch_count(const fi_handle* h);
/* Per-kernel CUDA-event timing of this handle's launches: enable = 1 on,
 * 0 off, -1 reset the totals.  fi_profile_read returns total milliseconds
 * and launch counts for kernel ids 0..n-1: 0 flexure, 1 rows_fwd,
 * 2 cols_hartley, 3 rows_inv, 4 conv_rows_fwd, 5 conv_cols, 6 conv_rows_inv,
 * 7 rk_stage, 8 rk_final, 9 upd_begin, 10 upd_masks, 11 upd_litho,
 * 12 upd_load, 13 upd_end. */
int fi_profile(fi_handle* h, int enable);
/* Step-engine phase timestamps (%globaltimer, ns) of the first RK4 step of
 * the last update, taken by block 0 at every phase and sub-phase boundary
 * (up to 256): the first call enables tracing (for updates launched after
 * it: a CUDA graph captured earlier keeps running untraced), later calls
 * copy up to n timestamps into `out`. */
int fi_engine_trace(fi_handle* h, unsigned long long* out, int n);
int fi_profile_read(fi_handle* h, double* ms, long long* counts, int n);

const char* fi_last_error(const fi_handle* h);
int fi_version(void);

#ifdef __cplusplus
}
#endif
#endif
