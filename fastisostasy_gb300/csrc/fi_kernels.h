// fi_kernels.h — host-side launchers of the LV-ELVA device kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fi_common.cuh"

namespace fi {

// Coefficients of the flexure stencil (calc_lvelva, src/lv_elva.f90:95-113).
struct FlexCoef {
    double nu, one_minus_nu;
    double coef_mantle;            // -g*rho_m in true-stage mode (mantle anomaly at the stage state), else 0
    double inv_dx, inv_2dx, inv_dx2, inv_dy, inv_2dy, inv_dy2;
    const double* dxm;             // per-cell dx*K, or null for uniform spacing
    const double* dym;
};

// The same coefficients rounded to float (mixed form, uniform spacing).
struct FlexCoefF {
    float nu, one_minus_nu, coef_mantle, inv_dx, inv_2dx, inv_dx2, inv_dy, inv_2dy, inv_dy2;
};

inline FlexCoefF flex_coef_f32(const FlexCoef& c)
{
    FlexCoefF f;
    f.nu = (float)c.nu;
    f.one_minus_nu = (float)c.one_minus_nu;
    f.coef_mantle = (float)c.coef_mantle;
    f.inv_dx = (float)c.inv_dx;
    f.inv_2dx = (float)c.inv_2dx;
    f.inv_dx2 = (float)c.inv_dx2;
    f.inv_dy = (float)c.inv_dy;
    f.inv_2dy = (float)c.inv_2dy;
    f.inv_dy2 = (float)c.inv_dy2;
    return f;
}

// One FFT length: factorisation + twiddle tables in both precisions.
struct FftLen {
    FftDesc d;
    const double2* tw64;    // exp(-2 pi i t / n), t < n
    const float2* tw32;
};

// A real 2-D transform layout: rows of nx reals -> nx/2+1 complex, pitch sp.
struct Plan2D {
    int nx, ny, h, sp;      // h = nx/2, sp = spectrum row pitch (complex elements)
    FftLen row;             // length h complex
    FftLen col;             // length ny complex
    const double2* rtw64;   // exp(-2 pi i k / nx), k <= h
    const float2* rtw32;
    int rb = 0, cb = 0;     // rows per row-transform block, columns per column-transform block (0: default)
    int rt = 0, ct = 0;     // threads per row- / column-transform block (0: default)
};

// The RHS launchers take an optional device flag: when it points at 0 every
// block returns at once (device-side skipping inside a graph loop).  The
// mixed-form flexure can take the state as a float pair y = whi + wlo
// (uniform spacing, no mantle term), which keeps it free of FP64 work.
template <typename T>
void launch_flexure(const double* y, const double* wref, const T* q0, const uint8_t* mask, const T* D,
                    const T* inv2eta, T* f, int nx, int ny, const FlexCoef& c, cudaStream_t s,
                    const int* gate = nullptr, const float* whi = nullptr, const float* wlo = nullptr);

// Mixed-form RK4 stage RHS (uniform spacing, true stages): the stage state
// x + (a h spy) (rprev - corner mean) from the float pair of x and the raw
// RHS of the previous stage (null at the first stage); the mantle term takes
// dxw = (xhi - w_ref,hi) + (xlo - w_ref,lo) per cell; h is read from the
// control block.  With a gate, every block returns at once when it is 0.
void launch_flexure_stage(const float* whi, const float* wlo, const float* rprev, const float* dxw, const float* q0,
                          const uint8_t* mask, const float* D, const float* inv2eta, float* f, int nx, int ny,
                          const FlexCoef& c, const Ctl* ctl, double a, double spy, cudaStream_t s,
                          const int* gate = nullptr);

template <typename T>
void launch_rows_fwd(const T* in, int in_pitch, int in_width, int nrows_in, typename vec2<T>::type* S,
                     const Plan2D& p, cudaStream_t s, const int* gate = nullptr);

template <typename T>
void launch_cols_hartley(typename vec2<T>::type* S, const T* mA, const T* mB, int even, const Plan2D& p,
                         cudaStream_t s, const int* gate = nullptr);

template <typename T>
void launch_rows_inv(const typename vec2<T>::type* S, T* out, const Plan2D& p, double scale, cudaStream_t s,
                     const int* gate = nullptr);

// Convolution: columns forward (rows >= nrows_in are zero), multiply by the
// kernel spectrum K (same layout as S), inverse; only rows listed in
// out_rows are written back (compacted to rows 0..n_out-1 of S).
template <typename T>
void launch_cols_conv(typename vec2<T>::type* S, const typename vec2<T>::type* K, int nrows_in,
                      const int* out_rows, int n_out, const Plan2D& p, cudaStream_t s);

template <typename T>
void launch_cols_fwd(typename vec2<T>::type* S, int nrows_in, const Plan2D& p, cudaStream_t s);

// inverse rows of the compacted convolution spectrum, crop + corner values
template <typename T>
void launch_conv_rows_inv(const typename vec2<T>::type* S, int n_out, double* out, int nx, int ny, int i_off,
                          double* corners, int corner_row0, int corner_row1, int corner_col1, const Plan2D& p,
                          double scale, cudaStream_t s);

}  // namespace fi
