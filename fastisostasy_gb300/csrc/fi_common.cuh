// fi_common.cuh — shared types and device helpers for the LV-ELVA kernels.
//
// Grid layout everywhere: a padded field (nx, ny) is stored with x fastest
// (the reference's Fortran column-major layout), element (i, j) at
// j*nx + i.  State fields are double; the transform/stencil pipeline runs in
// the "field type" T (double for the plain form, float for the mixed form).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fi {

template <typename T> struct vec2;
template <> struct vec2<float> { typedef float2 type; };
template <> struct vec2<double> { typedef double2 type; };

template <typename T> __host__ __device__ __forceinline__ typename vec2<T>::type mk2(T a, T b)
{
    typename vec2<T>::type r;
    r.x = a;
    r.y = b;
    return r;
}

template <typename C2> __device__ __forceinline__ C2 cmul(C2 a, C2 b)
{
    C2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// a * conj(b)
template <typename C2> __device__ __forceinline__ C2 cmulc(C2 a, C2 b)
{
    C2 r;
    r.x = a.x * b.x + a.y * b.y;
    r.y = a.y * b.x - a.x * b.y;
    return r;
}
template <typename C2> __device__ __forceinline__ C2 cadd(C2 a, C2 b) { a.x += b.x; a.y += b.y; return a; }
template <typename C2> __device__ __forceinline__ C2 csub(C2 a, C2 b) { a.x -= b.x; a.y -= b.y; return a; }

// Factorisation of one FFT length; lengths up to 4096 and radices from
// {8, 4, 2, 3, 5, 7} plus generic odd primes.
struct FftDesc {
    int n;
    int nf;
    int fac[16];
};

// Per-domain control block of the time integrator (device resident).
struct Ctl {
    double t, dt, tf, h;       // ode%t, ode%dt, target time, current step size
    double tol, err;           // last adaptive tolerance / error norm
    double bsl, V_af, V_den, V_pov, deltaV, dbsl_total, A_ocean;   // barystatic bookkeeping
    double red[8];             // scratch results of grid reductions
    int done;                  // t >= tf for the current update
    int accepted;              // last adaptive attempt accepted
    int rhs_valid;             // device Tsit5 loop: raw[0] holds the RHS of the current state
    int status;                // FI_* error code raised on the device
    int bsl_method;
    int need_rhs;              // device Tsit5 loop: gate of the RHS kernels for this attempt
    int have_rhs;              // device Tsit5 loop: an RHS was evaluated during this update
    int loop_iter;             // device Tsit5 loop: attempts during this update
    int active;                // device Tsit5 loop: this attempt runs (gate of the stage RHS)
    int plain;                 // methods 0-2: stage outputs are the rate itself (no corner mean, no sec/yr)
    long long n_accept, n_reject, n_rhs, n_attempt;
    // step-control limits (adaptive methods): a rejection that halves dt
    // below dt_min, or more than max_reject rejections within one update,
    // fails the update with ST_STEP; rej0 = n_reject when the update began
    double dt_min;
    long long max_reject, rej0;
    unsigned int counter[8];   // last-block arrival counters of grid reductions
};

// status codes (mirrors include/fi_gpu.h)
enum { ST_OK = 0, ST_NAN = 1, ST_LARGE = 2, ST_STEP = 3, ST_TIMEOUT = 4 };

__device__ __forceinline__ double corner_mean(const double c00, const double cnn, const double c0n,
                                              const double cn0)
{
    // apply_zerobc_at_corners: 0.25*(x(1,1) + x(nx,ny) + x(1,ny) + x(nx,1))
    return 0.25 * (((c00 + cnn) + c0n) + cn0);
}

template <typename T>
__device__ __forceinline__ double corner_mean_of(const T* a, int nx, int ny)
{
    const size_t last = (size_t)(ny - 1) * nx;
    return corner_mean((double)a[0], (double)a[last + nx - 1], (double)a[last], (double)a[nx - 1]);
}

}  // namespace fi
