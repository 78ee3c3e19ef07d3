// fi_state.h — device pointers and launchers of the sea-level / integrator
// kernels (double precision state).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fi_common.cuh"

namespace fi {

// Everything the per-cell update kernels touch for one domain.
struct Dom {
    int nx, ny;
    size_t n;
    int i0, j0, nxi, nyi;              // 0-based crop origin and ice-grid size
    int interactive;
    double rho_ice, rho_w, rho_m, rho_l, g, Vden, spy;
    double rho_sw_over_ice, rho_ice_over_sw;
    const double* A;
    const double* K2;                  // K**2
    const uint8_t* mactive;
    // reference state
    const double *z_bed_ref, *Hice_ref, *Haf_ref, *z_ss_ref, *we_ref, *w_ref;
    // current state
    double *z_bed, *w, *wout, *we, *Haf, *Hice, *z_ss, *dz_ss, *dwdt, *x;
    double *c_ice, *c_sw, *c_litho, *c_mantle, *c_load, *c_full, *mass;
    uint8_t *m_ocean, *m_grounded, *m_cont;
    Ctl* ctl;
    double* partials;                  // >= reduce_blocks(n) * 4 doubles
    double *ts_x2, *ts_dx;             // Tsit5 attempt: x2 and x2 - x1 (dt_method 2 only)
    float *whi, *wlo;                  // mixed Tsit5: now%w as a float pair (w = whi + wlo), else null
};

int reduce_blocks(size_t n);
void upd_begin(const Dom& d, const double* H_ice, cudaStream_t s);
template <typename T> void upd_masks(const Dom& d, T* conv_in, cudaStream_t s);
template <typename T>
void upd_litho(const Dom& d, const double* we_raw, const double* corners, int we_mode, T* conv_in, cudaStream_t s);
template <typename T>
void upd_load(const Dom& d, const double* dz_raw, const double* corners, int dz_mode, T* q0, int stage_mode,
              int run_integrator, cudaStream_t s);
void set_args(Ctl* c, double tf, double bsl, double A_ocean, int method, int write_bsl, cudaStream_t s);
void step_begin(Ctl* c, int kind, cudaStream_t s);
void step_end(Ctl* c, cudaStream_t s);
// device-side Tsit5 attempt loop (body of a CUDA graph WHILE node)
void ts_loop_begin(Ctl* c, cudaStream_t s);
void ts_attempt_begin(Ctl* c, int max_iter, cudaStream_t s);
// fsal: true stages (keep the cached first-stage RHS after an accept);
// more_out != NULL: write the loop condition there instead of `loop`
void ts_attempt_end(Ctl* c, cudaGraphConditionalHandle loop, cudaStream_t s, int fsal = 0, int* more_out = nullptr);
// true-stage Tsit5 (Dormand-Prince 5(4), FSAL): stage outputs k_0..k_6
template <typename T> struct DPRaw {
    const T* p[7];
};
template <typename T>
void dp_stage(const Ctl* c, double* y, const double* x, const DPRaw<T>& r, int i, int nx, int ny, double spy,
              cudaStream_t s);
template <typename T> void dp_err(const Dom& d, const DPRaw<T>& r, double atol, double rtol, cudaStream_t s);
template <typename T> void fsal_copy(const Ctl* c, T* k0, const T* k6, size_t n, cudaStream_t s);
template <typename T>
void rk_stage(const Ctl* c, double* y, const double* x, const T* raw, double a, int nx, int ny, double spy,
              cudaStream_t s);
template <typename T>
void rk4_final(Ctl* c, double* x, double* w, const T* r1, const T* r2, const T* r3, const T* r4, int nx, int ny,
               double spy, cudaStream_t s);
// true-stage Tsit5, mixed form: stage state i as a float pair (yhi, ylo) with
// its dxw, x2 in FP64 at stage 6 (x2 non-null); the commit takes the
// stage-6 pair into the pair of x
void dp_stage_pair(const Ctl* c, const float* xhi, const float* xlo, const float* wrhi, const float* wrlo, float* yhi,
                   float* ylo, float* ydw, double* x2, const double* x, const DPRaw<float>& r, int i, int nx, int ny,
                   double spy, cudaStream_t s);
void ts_commit_tpair(const Dom& d, float* xhi, float* xlo, float* xdw, const float* yhi, const float* ylo,
                     const float* ydw, cudaStream_t s);
// mixed RK4 combination that also advances the float pair xhi + xlo of x and
// dxw = (xhi - wrhi) + (xlo - wrlo)
void rk4_final_pair(Ctl* c, double* x, double* w, float* xhi, float* xlo, const float* wrhi, const float* wrlo,
                    float* dxw, const float* r1, const float* r2, const float* r3, const float* r4, int nx, int ny,
                    double spy, cudaStream_t s);
template <typename T>
void euler_final(const Ctl* c, double* x, double* w, const T* r1, int nx, int ny, double spy, cudaStream_t s);
template <typename T> void ts_max(const Dom& d, const T* raw, double atol, double rtol, cudaStream_t s);
template <typename T>
void ts_err(const Dom& d, const T* raw, double q, double dt_max, cudaStream_t s);
template <typename T> void ts_commit(const Dom& d, const T* raw, cudaStream_t s);
// Mixed form with now%w's float pair (d.whi/d.wlo): tolerance, error norm
// and decision in one pass, then the commit of an accepted attempt.
void ts_fused(const Dom& d, const float* raw, double atol, double rtol, double q, double dt_max,
              cudaStream_t s);
void ts_commit_pair(const Dom& d, const float* raw, cudaStream_t s);
// have_rhs < 0: read it from the control block (device Tsit5 loop)
template <typename T> void upd_end(const Dom& d, const T* raw_last, int have_rhs, cudaStream_t s);
void gather(const double* const* src, const uint8_t* const* msrc, int nf, int nm, const Dom& d, double* out,
            cudaStream_t s);
// the same with the masks as bytes into mout (nm * nxi * nyi bytes)
void gather_bytes(const double* const* src, const uint8_t* const* msrc, int nf, int nm, const Dom& d, double* out,
                  uint8_t* mout, cudaStream_t s);
void out2in(double* dst, const double* src, const Dom& d, double background, int keep_outside, cudaStream_t s);
void state_diag(double* z_ss, const double* zss_base, const double* dz_ss, double bsl, const double* z_bed,
                const double* Hice, double* Haf, uint8_t* mo, uint8_t* mg, uint8_t* mc, size_t n,
                double rho_sw_over_ice, cudaStream_t s);
template <typename T> void rhs_finish(double* out, const T* raw, int nx, int ny, double spy, cudaStream_t s);
// LLRA / LV-ELRA (methods 0-2): equilibrium displacement and relaxation rate
void weq_local(double* weq, const double* c_load, double rho_m, int zero, size_t n, cudaStream_t s);
template <typename T> void elra_load(T* in, const double* c_load, const double* K2, double g, size_t n, cudaStream_t s);
void weq_elra(double* weq, const double* raw, const double* corners, int nx, int ny, cudaStream_t s);
template <typename T>
void relax_rate(T* out, const double* y, const double* weq, double tau, size_t n, const int* gate, cudaStream_t s);
void sub_corner(double* out, const double* raw, const double* corners, size_t n, cudaStream_t s);
template <typename T> void cast_from_double(T* dst, const double* src, size_t n, cudaStream_t s);
template <typename T> void q0_from_cf(T* q0, const double* cf, const uint8_t* mask, double g, size_t n, cudaStream_t s);

}  // namespace fi
