// fi_rhs.cu — the LV-ELVA viscous-rate pipeline and the FFT convolution
// passes (calc_lvelva, src/lv_elva.f90:31-126; precomputed_fftconvolution,
// src/convolutions.f90:59-91).
//
// RHS = four kernels:
//   k_flexure      finite-difference flexure moments and load -> f      (one pass over the grid)
//   k_rows_fwd     real FFT of every row of f -> half spectrum S
//   k_cols_hartley column FFT, multiply by 1/(kappa R) in the Hartley basis, inverse column FFT
//   k_rows_inv     inverse real FFT of the rows, scaled by 1/(nx*ny) -> raw
// The corner boundary condition and the sec_per_year factor are applied by
// whichever kernel consumes raw (it reads the four corner values).
//
// The reference transforms with FFTW's separable DHT.  The Hartley
// coefficients are formed from the DFT in the column kernel,
//   H[k,l] = Re F[k,-l] - Im F[k,l],
// multiplied by m = 1/(kappa R) at all four (+-k, +-l), and turned back into
// the DFT of DHT^-1(m H); when m is even in both indices this reduces to
// F' = m F (flag `even`).
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "fi_fft.cuh"

#include "fi_batch.h"
#include "fi_kernels.h"

namespace fi {

template <typename T> __device__ __forceinline__ const typename vec2<T>::type* twp(const FftLen& L);
template <> __device__ __forceinline__ const double2* twp<double>(const FftLen& L) { return L.tw64; }
template <> __device__ __forceinline__ const float2* twp<float>(const FftLen& L) { return L.tw32; }
template <typename T> __device__ __forceinline__ const typename vec2<T>::type* rtwp(const Plan2D& p);
template <> __device__ __forceinline__ const double2* rtwp<double>(const Plan2D& p) { return p.rtw64; }
template <> __device__ __forceinline__ const float2* rtwp<float>(const Plan2D& p) { return p.rtw32; }

// Raise a kernel's dynamic shared-memory limit when a larger launch needs it
// (the limit belongs to the kernel and is shared by every handle, so it only
// ever grows).
template <typename K> static void set_smem(K kern, size_t bytes)
{
    static std::mutex mu;
    static const void* fn[64];
    static size_t done[64];
    static int nfn = 0;
    if (bytes <= 48 * 1024) return;
    std::lock_guard<std::mutex> lk(mu);
    const void* key = (const void*)kern;
    for (int i = 0; i < nfn; ++i)
        if (fn[i] == key) {
            if (done[i] >= bytes) return;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            done[i] = bytes;
            return;
        }
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (nfn < 64) { fn[nfn] = key; done[nfn] = bytes; ++nfn; }
}

// ---------------------------------------------------------------------------
// Flexure stencil.  Tile TX x TY outputs with a halo of 2; the first-level
// differences are taken on the double state, then rounded to T.
// ---------------------------------------------------------------------------
constexpr int TX = 32, TY = 8, RX = TX + 4, RY = TY + 4;

template <typename T>
__device__ __forceinline__ void flexure_body(const double* __restrict__ y, const double* __restrict__ wref, const T* __restrict__ q0,
          const uint8_t* __restrict__ mask, const T* __restrict__ D, const T* __restrict__ inv2eta,
          T* __restrict__ f, int nx, int ny, FlexCoef c, int bx, int by)
{
    __shared__ double ys[RY][RX];
    __shared__ T wx[RY][RX];
    __shared__ T Mxx[RY][RX];
    __shared__ T Myy[RY][RX];
    __shared__ T Mxy[RY][RX];
    __shared__ T Mxyx[RY][RX];
    const int tid = threadIdx.x + TX * threadIdx.y;
    const int i0 = bx * TX, j0 = by * TY;
    const bool uni = (c.dxm == nullptr);

    // per-cell spacing accessors (uniform fast path)
    auto idx1 = [&](int i, int j) -> double { return uni ? c.inv_dx : 1.0 / c.dxm[(size_t)j * nx + i]; };
    auto idx2h = [&](int i, int j) -> double { return uni ? c.inv_2dx : 1.0 / (2 * c.dxm[(size_t)j * nx + i]); };
    auto idxx = [&](int i, int j) -> double {
        if (uni) return c.inv_dx2;
        const double d = c.dxm[(size_t)j * nx + i];
        return 1.0 / (d * d);
    };
    auto idy1 = [&](int i, int j) -> double { return uni ? c.inv_dy : 1.0 / c.dym[(size_t)j * nx + i]; };
    auto idy2h = [&](int i, int j) -> double { return uni ? c.inv_2dy : 1.0 / (2 * c.dym[(size_t)j * nx + i]); };
    auto idyy = [&](int i, int j) -> double {
        if (uni) return c.inv_dy2;
        const double d = c.dym[(size_t)j * nx + i];
        return 1.0 / (d * d);
    };

    for (int e = tid; e < RX * RY; e += TX * TY) {
        const int lx = e % RX, ly = e / RX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        ys[ly][lx] = (gi >= 0 && gi < nx && gj >= 0 && gj < ny) ? y[(size_t)gj * nx + gi] : 0.0;
    }
    __syncthreads();
    // w_x on lx in [1, RX-1), all rows
    for (int e = tid; e < RX * RY; e += TX * TY) {
        const int lx = e % RX, ly = e / RX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        if (lx < 1 || lx >= RX - 1 || gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
        double v;
        if (gi == 0) v = (ys[ly][lx + 1] - ys[ly][lx]) * idx1(gi, gj);
        else if (gi == nx - 1) v = (ys[ly][lx] - ys[ly][lx - 1]) * idx1(gi, gj);
        else v = (ys[ly][lx + 1] - ys[ly][lx - 1]) * idx2h(gi, gj);
        wx[ly][lx] = (T)v;
    }
    __syncthreads();
    // level 1: w_xy, w_xx, w_yy -> moments, on lx, ly in [1, R-1)
    for (int e = tid; e < RX * RY; e += TX * TY) {
        const int lx = e % RX, ly = e / RX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        if (lx < 1 || lx >= RX - 1 || ly < 1 || ly >= RY - 1 || gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
        T wxy;
        if (gj == 0) wxy = (wx[ly + 1][lx] - wx[ly][lx]) * (T)idy1(gi, gj);
        else if (gj == ny - 1) wxy = (wx[ly][lx] - wx[ly - 1][lx]) * (T)idy1(gi, gj);
        else wxy = (wx[ly + 1][lx] - wx[ly - 1][lx]) * (T)idy2h(gi, gj);
        double dxx, dyy;
        if (gi == 0) dxx = ((ys[ly][lx + 2] - 2 * ys[ly][lx + 1]) + ys[ly][lx]) * idxx(0, gj);
        else if (gi == nx - 1) dxx = ((ys[ly][lx] - 2 * ys[ly][lx - 1]) + ys[ly][lx - 2]) * idxx(0, gj);
        else dxx = ((ys[ly][lx + 1] - 2 * ys[ly][lx]) + ys[ly][lx - 1]) * idxx(gi, gj);
        if (gj == 0) dyy = ((ys[ly + 2][lx] - 2 * ys[ly + 1][lx]) + ys[ly][lx]) * idyy(gi, 0);
        else if (gj == ny - 1) dyy = ((ys[ly][lx] - 2 * ys[ly - 1][lx]) + ys[ly - 2][lx]) * idyy(gi, gj);
        else dyy = ((ys[ly + 1][lx] - 2 * ys[ly][lx]) + ys[ly - 1][lx]) * idyy(gi, gj);
        const T wxx = (T)dxx, wyy = (T)dyy;
        const T Dl = D[(size_t)gj * nx + gi];
        const T nu = (T)c.nu;
        Mxx[ly][lx] = -Dl * (wxx + nu * wyy);
        Myy[ly][lx] = -Dl * (wyy + nu * wxx);
        Mxy[ly][lx] = (-Dl * (T)c.one_minus_nu) * wxy;
    }
    __syncthreads();
    // d/dx of Mxy on lx in [2, RX-2), ly in [1, RY-1)
    for (int e = tid; e < RX * RY; e += TX * TY) {
        const int lx = e % RX, ly = e / RX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        if (lx < 2 || lx >= RX - 2 || ly < 1 || ly >= RY - 1 || gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
        T v;
        if (gi == 0) v = (Mxy[ly][lx + 1] - Mxy[ly][lx]) * (T)idx1(gi, gj);
        else if (gi == nx - 1) v = (Mxy[ly][lx] - Mxy[ly][lx - 1]) * (T)idx1(gi, gj);
        else v = (Mxy[ly][lx + 1] - Mxy[ly][lx - 1]) * (T)idx2h(gi, gj);
        Mxyx[ly][lx] = v;
    }
    __syncthreads();
    {
        const int lx = threadIdx.x + 2, ly = threadIdx.y + 2;
        const int gi = i0 + threadIdx.x, gj = j0 + threadIdx.y;
        if (gi < nx && gj < ny) {
            T mxy_xy, mx_xx, my_yy;
            if (gj == 0) mxy_xy = (Mxyx[ly + 1][lx] - Mxyx[ly][lx]) * (T)idy1(gi, gj);
            else if (gj == ny - 1) mxy_xy = (Mxyx[ly][lx] - Mxyx[ly - 1][lx]) * (T)idy1(gi, gj);
            else mxy_xy = (Mxyx[ly + 1][lx] - Mxyx[ly - 1][lx]) * (T)idy2h(gi, gj);
            if (gi == 0) mx_xx = ((Mxx[ly][lx + 2] - (T)2 * Mxx[ly][lx + 1]) + Mxx[ly][lx]) * (T)idxx(0, gj);
            else if (gi == nx - 1) mx_xx = ((Mxx[ly][lx] - (T)2 * Mxx[ly][lx - 1]) + Mxx[ly][lx - 2]) * (T)idxx(0, gj);
            else mx_xx = ((Mxx[ly][lx + 1] - (T)2 * Mxx[ly][lx]) + Mxx[ly][lx - 1]) * (T)idxx(gi, gj);
            if (gj == 0) my_yy = ((Myy[ly + 2][lx] - (T)2 * Myy[ly + 1][lx]) + Myy[ly][lx]) * (T)idyy(gi, 0);
            else if (gj == ny - 1) my_yy = ((Myy[ly][lx] - (T)2 * Myy[ly - 1][lx]) + Myy[ly - 2][lx]) * (T)idyy(gi, gj);
            else my_yy = ((Myy[ly + 1][lx] - (T)2 * Myy[ly][lx]) + Myy[ly - 1][lx]) * (T)idyy(gi, gj);
            const size_t e = (size_t)gj * nx + gi;
            T p = (T)0;
            if (mask[e]) {
                double pm = (double)q0[e];
                if (wref) pm += c.coef_mantle * (ys[ly][lx] - wref[e]);
                p = (T)pm;
            }
            f[e] = (((p + mx_xx) + (T)2 * mxy_xy) + my_yy) * inv2eta[e];
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(TX* TY)
k_flexure(const double* __restrict__ y, const double* __restrict__ wref, const T* __restrict__ q0,
          const uint8_t* __restrict__ mask, const T* __restrict__ D, const T* __restrict__ inv2eta,
          T* __restrict__ f, int nx, int ny, FlexCoef c, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    flexure_body<T>(y, wref, q0, mask, D, inv2eta, f, nx, ny, c, blockIdx.x, blockIdx.y);
}

// Mixed form, uniform spacing.  The only double work per cell is the pair of
// forward differences of the double state, dX = y[i+1]-y[i] and
// dY = y[j+1]-y[j] (taken before rounding to float, so the second
// differences keep the small curvature of a large smooth field), and the
// mantle term y - w_ref.  Central and second differences are rebuilt
// exactly from them: y[i+1]-y[i-1] = dX[i]+dX[i-1],
// y[i+1]-2y[i]+y[i-1] = dX[i]-dX[i-1].
// HILO: the state arrives as a float pair y = hi + lo (whi, wlo) instead of
// doubles, and the first differences are (hi[i+1]-hi[i]) + (lo[i+1]-lo[i]),
// all in float (no mantle term in this form).
template <bool HILO>
__device__ __forceinline__ void flexure_f32_body(const double* __restrict__ y, const double* __restrict__ wref,
                                                 const float* __restrict__ q0, const uint8_t* __restrict__ mask,
                                                 const float* __restrict__ D, const float* __restrict__ inv2eta,
                                                 float* __restrict__ f, int nx, int ny, FlexCoefF c, int bx, int by,
                                                 const float* __restrict__ whi = nullptr,
                                                 const float* __restrict__ wlo = nullptr)
{
    __shared__ double ys[HILO ? 1 : RY][HILO ? 1 : RX];
    __shared__ float yh[HILO ? RY : 1][HILO ? RX : 1];
    __shared__ float yl[HILO ? RY : 1][HILO ? RX : 1];
    __shared__ float dX[RY][RX];
    __shared__ float dY[RY][RX];
    __shared__ float Wx[RY][RX];
    __shared__ float Mxx[RY][RX];
    __shared__ float Myy[RY][RX];
    __shared__ float Mxy[RY][RX];
    __shared__ float Mxyx[RY][RX];
    __shared__ float Ds[RY][RX];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = bx * TX - 2, j0 = by * TY - 2;   // global index of lx = ly = 0
    // every global input is requested up front, so their latencies overlap:
    // this thread's output cell ...
    const int go_i = i0 + tx + 2, go_j = j0 + ty + 2;
    const bool own = go_i < nx && go_j < ny;
    const size_t eo = own ? (size_t)go_j * nx + go_i : 0;
    const uint8_t own_m = own ? mask[eo] : (uint8_t)0;
    const float own_q = own ? q0[eo] : 0.f, own_ie = own ? inv2eta[eo] : 0.f;
    // ... and the state and rigidity tiles with their halo
    for (int ly = ty; ly < RY; ly += TY)
        for (int lx = tx; lx < RX; lx += TX) {
            const int gi = i0 + lx, gj = j0 + ly;
            const bool in = gi >= 0 && gi < nx && gj >= 0 && gj < ny;
            Ds[ly][lx] = in ? D[(size_t)gj * nx + gi] : 0.f;
            if constexpr (HILO) {
                yh[ly][lx] = in ? whi[(size_t)gj * nx + gi] : 0.f;
                yl[ly][lx] = in ? wlo[(size_t)gj * nx + gi] : 0.f;
            } else {
                ys[ly][lx] = in ? y[(size_t)gj * nx + gi] : 0.0;
            }
        }
    __syncthreads();
    for (int ly = ty; ly < RY; ly += TY)
        for (int lx = tx; lx < RX; lx += TX) {
            if constexpr (HILO) {
                if (lx < RX - 1) dX[ly][lx] = (yh[ly][lx + 1] - yh[ly][lx]) + (yl[ly][lx + 1] - yl[ly][lx]);
                if (ly < RY - 1) dY[ly][lx] = (yh[ly + 1][lx] - yh[ly][lx]) + (yl[ly + 1][lx] - yl[ly][lx]);
            } else {
                if (lx < RX - 1) dX[ly][lx] = (float)(ys[ly][lx + 1] - ys[ly][lx]);
                if (ly < RY - 1) dY[ly][lx] = (float)(ys[ly + 1][lx] - ys[ly][lx]);
            }
        }
    __syncthreads();
    for (int ly = ty; ly < RY; ly += TY)
        for (int lx = tx + 1; lx < RX - 1; lx += TX) {
            const int gi = i0 + lx, gj = j0 + ly;
            if (gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
            float v;
            if (gi == 0) v = dX[ly][lx] * c.inv_dx;
            else if (gi == nx - 1) v = dX[ly][lx - 1] * c.inv_dx;
            else v = (dX[ly][lx] + dX[ly][lx - 1]) * c.inv_2dx;
            Wx[ly][lx] = v;
        }
    __syncthreads();
    for (int ly = ty + 1; ly < RY - 1; ly += TY)
        for (int lx = tx + 1; lx < RX - 1; lx += TX) {
            const int gi = i0 + lx, gj = j0 + ly;
            if (gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
            float wxy, wxx, wyy;
            if (gj == 0) wxy = (Wx[ly + 1][lx] - Wx[ly][lx]) * c.inv_dy;
            else if (gj == ny - 1) wxy = (Wx[ly][lx] - Wx[ly - 1][lx]) * c.inv_dy;
            else wxy = (Wx[ly + 1][lx] - Wx[ly - 1][lx]) * c.inv_2dy;
            if (gi == 0) wxx = (dX[ly][lx + 1] - dX[ly][lx]) * c.inv_dx2;
            else if (gi == nx - 1) wxx = (dX[ly][lx - 1] - dX[ly][lx - 2]) * c.inv_dx2;
            else wxx = (dX[ly][lx] - dX[ly][lx - 1]) * c.inv_dx2;
            if (gj == 0) wyy = (dY[ly + 1][lx] - dY[ly][lx]) * c.inv_dy2;
            else if (gj == ny - 1) wyy = (dY[ly - 1][lx] - dY[ly - 2][lx]) * c.inv_dy2;
            else wyy = (dY[ly][lx] - dY[ly - 1][lx]) * c.inv_dy2;
            const float Dl = Ds[ly][lx];
            Mxx[ly][lx] = -Dl * (wxx + c.nu * wyy);
            Myy[ly][lx] = -Dl * (wyy + c.nu * wxx);
            Mxy[ly][lx] = (-Dl * c.one_minus_nu) * wxy;
        }
    __syncthreads();
    for (int ly = ty + 1; ly < RY - 1; ly += TY)
        for (int lx = tx + 2; lx < RX - 2; lx += TX) {
            const int gi = i0 + lx, gj = j0 + ly;
            if (gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
            float v;
            if (gi == 0) v = (Mxy[ly][lx + 1] - Mxy[ly][lx]) * c.inv_dx;
            else if (gi == nx - 1) v = (Mxy[ly][lx] - Mxy[ly][lx - 1]) * c.inv_dx;
            else v = (Mxy[ly][lx + 1] - Mxy[ly][lx - 1]) * c.inv_2dx;
            Mxyx[ly][lx] = v;
        }
    __syncthreads();
    const int lx = tx + 2, ly = ty + 2;
    const int gi = i0 + lx, gj = j0 + ly;
    if (gi >= nx || gj >= ny) return;
    float mxy_xy, mx_xx, my_yy;
    if (gj == 0) mxy_xy = (Mxyx[ly + 1][lx] - Mxyx[ly][lx]) * c.inv_dy;
    else if (gj == ny - 1) mxy_xy = (Mxyx[ly][lx] - Mxyx[ly - 1][lx]) * c.inv_dy;
    else mxy_xy = (Mxyx[ly + 1][lx] - Mxyx[ly - 1][lx]) * c.inv_2dy;
    if (gi == 0) mx_xx = ((Mxx[ly][lx + 2] - 2.f * Mxx[ly][lx + 1]) + Mxx[ly][lx]) * c.inv_dx2;
    else if (gi == nx - 1) mx_xx = ((Mxx[ly][lx] - 2.f * Mxx[ly][lx - 1]) + Mxx[ly][lx - 2]) * c.inv_dx2;
    else mx_xx = ((Mxx[ly][lx + 1] - 2.f * Mxx[ly][lx]) + Mxx[ly][lx - 1]) * c.inv_dx2;
    if (gj == 0) my_yy = ((Myy[ly + 2][lx] - 2.f * Myy[ly + 1][lx]) + Myy[ly][lx]) * c.inv_dy2;
    else if (gj == ny - 1) my_yy = ((Myy[ly][lx] - 2.f * Myy[ly - 1][lx]) + Myy[ly - 2][lx]) * c.inv_dy2;
    else my_yy = ((Myy[ly + 1][lx] - 2.f * Myy[ly][lx]) + Myy[ly - 1][lx]) * c.inv_dy2;
    const size_t e = eo;
    float p = 0.f;
    if (own_m) {
        p = own_q;
        if constexpr (!HILO) {
            if (wref) p += c.coef_mantle * (float)(ys[ly][lx] - wref[e]);
        }
    }
    f[e] = (((p + mx_xx) + 2.f * mxy_xy) + my_yy) * own_ie;
}

// ---------------------------------------------------------------------------
// Flexure by column strips (mixed form, uniform spacing, the state as a
// float pair).  One warp task = SW output columns [SW g, SW g + SW) by `seg`
// output rows [seg s, seg s + seg): lane l holds column SW g - 2 + l and
// walks down the rows with the vertical stencil window in registers, taking
// x-neighbours by warp shuffles, so there is no shared memory and no block
// barrier.  Moments of row m are formed when input row m + 2 has been read,
// f of row o when moments of row o + 2 exist (the one-sided formulas of the
// first and last rows reach two rows further than the interior ones); the
// arithmetic is that of flexure_f32_body<true>, term by term.
// ---------------------------------------------------------------------------
constexpr int SW = 28;                     // output columns per warp task

__device__ __forceinline__ int strip_tasks(int nx, int ny, int seg)
{
    return ((nx + SW - 1) / SW) * ((ny + seg - 1) / seg);
}

// PAIR: the state as a float pair (whi + wlo), no mantle term; else the
// FP64 state y, its first differences taken in double and rounded (as
// flexure_f32_body<false>), and with wref the mantle term
// coef_mantle (y - wref) at masked cells.
// STG (with PAIR): an RK stage state y = x + sdf (rprev - cm) formed on the
// fly from the pair x = whi + wlo and the previous stage's raw RHS rprev
// (null at the first stage), with the mantle term
// coef_mantle (dxw + sdf (rprev - cm)) at masked cells, where
// dxw = (whi - w_ref,hi) + (wlo - w_ref,lo) is kept per cell beside the pair:
// the arithmetic of the step engine's phase A, term by term, and no FP64
// instruction.  (Loading every field one row ahead, as the state already is,
// takes 78 registers instead of 64 and ran 35 % slower at 2048^2: the walk
// is bound by warps in flight, not by the distance of each warp's loads.)
template <bool PAIR, bool STG = false>
__device__ __forceinline__ void flexure_strip(const float* __restrict__ whi, const float* __restrict__ wlo,
                                              const float* __restrict__ q0, const uint8_t* __restrict__ mask,
                                              const float* __restrict__ D, const float* __restrict__ inv2eta,
                                              float* __restrict__ f, int nx, int ny, const FlexCoefF& c, int seg,
                                              int task, const double* __restrict__ y = nullptr,
                                              const double* __restrict__ wref = nullptr,
                                              const float* __restrict__ rprev = nullptr, float sdf = 0.f,
                                              float cmdf = 0.f, const float* __restrict__ dxw = nullptr)
{
    static_assert(PAIR || !STG, "stage states are formed from the float pair");
    const unsigned FULL = 0xffffffffu;
    const int ncg = (nx + SW - 1) / SW;
    const int g = task % ncg, sg = task / ncg;
    const int lane = (int)(threadIdx.x + threadIdx.y * blockDim.x) & 31;   // 1D or 32 x 8 blocks
    const int col = g * SW - 2 + lane;
    const bool cin = col >= 0 && col < nx;
    const bool outl = cin && lane >= 2 && lane < 2 + SW;
    const bool left = col == 0, right = col == nx - 1;
    const bool edge = g == 0 || g == ncg - 1;   // warp-uniform: a lane may sit on x = 0 or x = nx - 1
    const int o0 = sg * seg, o1 = min(o0 + seg, ny);
    const int cc = cin ? col : 0;
    float hp = 0.f, lp = 0.f;                           // pair of row r - 1
    float rp = 0.f;                                     // rprev of row r - 1 (STG)
    double yp = 0.0;                                    // FP64 state of row r - 1 (!PAIR)
    float Wx1 = 0.f, Wx2 = 0.f, Wx3 = 0.f;              // Wx of rows r-1, r-2, r-3
    float wxx1 = 0.f, wxx2 = 0.f;                       // wxx of rows r-1, r-2
    float dY1 = 0.f, dY2 = 0.f, dY3 = 0.f, dY4 = 0.f;   // dY of rows r-1 .. r-4 (dY_j = y_{j+1} - y_j)
    float My0 = 0.f, My1 = 0.f, My2 = 0.f, My3 = 0.f, My4 = 0.f;   // Myy of rows m .. m-4
    float Mq0 = 0.f, Mq1 = 0.f, Mq2 = 0.f, Mq3 = 0.f;              // Mxyx of rows m .. m-3
    float mx0 = 0.f, mx1 = 0.f, mx2 = 0.f;                         // mx_xx of rows m .. m-2
    // the next row's loads are issued one iteration ahead
    int r = o0 - 4;
    const bool stg = STG && rprev != nullptr;   // uniform
    auto ld_pair = [&](int rr, float& h, float& l, double& yy, float& rv) {
        if (cin && rr >= 0 && rr < ny) {
            const size_t e = (size_t)rr * nx + cc;
            if constexpr (PAIR) {
                h = __ldg(whi + e);
                l = __ldg(wlo + e);
                if (stg) rv = __ldg(rprev + e);
            } else {
                yy = __ldg(y + e);
            }
        } else {
            h = 0.f;
            l = 0.f;
            yy = 0.0;
            rv = 0.f;
        }
    };
    float hn = 0.f, ln = 0.f, rn = 0.f;
    double yn = 0.0;
    ld_pair(r, hn, ln, yn, rn);
    // the fields of input row rr that are used at rows m = rr - 2 (D) and
    // o = rr - 4 (mask, load, 1/(2 eta), and with STG dxw and rprev)
    auto ld_rest = [&](int rr, float& Dv, uint32_t& mv, float& qv, float& iev, float& dv, float& rov) {
        const int mm = rr - 2, oo = rr - 4;
        const bool mr = cin && mm >= 0 && mm < ny;
        Dv = mr ? __ldg(D + (size_t)mm * nx + cc) : 0.f;
        const bool orr = outl && oo >= o0 && oo < o1;
        const size_t ee = orr ? (size_t)oo * nx + cc : 0;
        mv = orr ? (uint32_t)__ldg(mask + ee) : 0u;
        qv = orr ? __ldg(q0 + ee) : 0.f;
        iev = orr ? __ldg(inv2eta + ee) : 0.f;
        if constexpr (STG) {
            dv = orr ? __ldg(dxw + ee) : 0.f;
            rov = (orr && stg) ? __ldg(rprev + ee) : 0.f;
        }
    };
    for (; r < o1 + 4; ++r) {
        const float h = hn, l = ln, rv = rn;
        const double yv = yn;
        ld_pair(r + 1, hn, ln, yn, rn);
        const int m = r - 2, o = r - 4;
        const bool orow = outl && o >= o0 && o < o1;
        const size_t eo = orow ? (size_t)o * nx + cc : 0;
        float Dm, oq, oie, od = 0.f, orv = 0.f;
        uint32_t om;
        if constexpr (STG) {
            ld_rest(r, Dm, om, oq, oie, od, orv);
        } else {
            const bool mrow = cin && m >= 0 && m < ny;
            Dm = mrow ? __ldg(D + (size_t)m * nx + cc) : 0.f;
            om = orow ? __ldg(mask + eo) : (uint8_t)0;
            oq = orow ? __ldg(q0 + eo) : 0.f;
            oie = orow ? __ldg(inv2eta + eo) : 0.f;
        }
        // row r: first differences, Wx, wxx
        float dX;
        if constexpr (PAIR) {
            const float hr = __shfl_down_sync(FULL, h, 1), lr = __shfl_down_sync(FULL, l, 1);
            dX = (hr - h) + (lr - l);
            if constexpr (STG) {
                const float rr = __shfl_down_sync(FULL, rv, 1);
                if (stg) dX += sdf * (rr - rv);
            }
        } else {
            const double yr = __shfl_down_sync(FULL, yv, 1);
            dX = (float)(yr - yv);
        }
        const float dXm = __shfl_up_sync(FULL, dX, 1);
        float Wx, wxx;
        if (edge) {
            const float dXp = __shfl_down_sync(FULL, dX, 1), dXmm = __shfl_up_sync(FULL, dX, 2);
            Wx = left ? dX * c.inv_dx : right ? dXm * c.inv_dx : (dX + dXm) * c.inv_2dx;
            wxx = left ? (dXp - dX) * c.inv_dx2 : right ? (dXm - dXmm) * c.inv_dx2 : (dX - dXm) * c.inv_dx2;
        } else {
            Wx = (dX + dXm) * c.inv_2dx;
            wxx = (dX - dXm) * c.inv_dx2;
        }
        float dYn;   // dY of row r - 1
        if constexpr (PAIR) {
            dYn = (h - hp) + (l - lp);
            if constexpr (STG) {
                if (stg) dYn += sdf * (rv - rp);
                rp = rv;
            }
        } else {
            dYn = (float)(yv - yp);
        }
        hp = h;
        lp = l;
        yp = yv;
        dY4 = dY3; dY3 = dY2; dY2 = dY1; dY1 = dYn;
        // moments of row m = r - 2 (Wx1..3 are still those of rows r-1..r-3)
        float wxy, wyy;
        if (m == 0) {
            wxy = (Wx1 - Wx2) * c.inv_dy;
            wyy = (dY1 - dY2) * c.inv_dy2;
        } else if (m == ny - 1) {
            wxy = (Wx2 - Wx3) * c.inv_dy;
            wyy = (dY3 - dY4) * c.inv_dy2;
        } else {
            wxy = (Wx1 - Wx3) * c.inv_2dy;
            wyy = (dY2 - dY3) * c.inv_dy2;
        }
        const float wxm = wxx2;
        const float Mxx = -Dm * (wxm + c.nu * wyy);
        const float Myy = -Dm * (wyy + c.nu * wxm);
        const float Mxy = (-Dm * c.one_minus_nu) * wxy;
        Wx3 = Wx2; Wx2 = Wx1; Wx1 = Wx;
        wxx2 = wxx1; wxx1 = wxx;
        // x-derivatives of the moments of row m
        const float Mxyp = __shfl_down_sync(FULL, Mxy, 1), Mxym = __shfl_up_sync(FULL, Mxy, 1);
        const float Mxxp = __shfl_down_sync(FULL, Mxx, 1), Mxxm = __shfl_up_sync(FULL, Mxx, 1);
        float Mxyx, mxx;
        if (edge) {
            const float Mxxp2 = __shfl_down_sync(FULL, Mxx, 2), Mxxm2 = __shfl_up_sync(FULL, Mxx, 2);
            Mxyx = left ? (Mxyp - Mxy) * c.inv_dx : right ? (Mxy - Mxym) * c.inv_dx : (Mxyp - Mxym) * c.inv_2dx;
            mxx = left ? ((Mxxp2 - 2.f * Mxxp) + Mxx) * c.inv_dx2
                : right ? ((Mxx - 2.f * Mxxm) + Mxxm2) * c.inv_dx2
                : ((Mxxp - 2.f * Mxx) + Mxxm) * c.inv_dx2;
        } else {
            Mxyx = (Mxyp - Mxym) * c.inv_2dx;
            mxx = ((Mxxp - 2.f * Mxx) + Mxxm) * c.inv_dx2;
        }
        My4 = My3; My3 = My2; My2 = My1; My1 = My0; My0 = Myy;
        Mq3 = Mq2; Mq2 = Mq1; Mq1 = Mq0; Mq0 = Mxyx;
        mx2 = mx1; mx1 = mx0; mx0 = mxx;
        // f of row o = m - 2
        if (orow) {
            float mxy_xy, my_yy;
            if (o == 0) {
                mxy_xy = (Mq1 - Mq2) * c.inv_dy;
                my_yy = ((My0 - 2.f * My1) + My2) * c.inv_dy2;
            } else if (o == ny - 1) {
                mxy_xy = (Mq2 - Mq3) * c.inv_dy;
                my_yy = ((My2 - 2.f * My3) + My4) * c.inv_dy2;
            } else {
                mxy_xy = (Mq1 - Mq3) * c.inv_2dy;
                my_yy = ((My1 - 2.f * My2) + My3) * c.inv_dy2;
            }
            float p = om ? oq : 0.f;
            if constexpr (!PAIR) {
                if (om && wref) p += c.coef_mantle * (float)(__ldg(y + eo) - __ldg(wref + eo));
            }
            if constexpr (STG) {
                if (om) {
                    float dy = od;
                    if (stg) dy += sdf * (orv - cmdf);
                    p = oq + c.coef_mantle * dy;
                }
            }
            f[eo] = (((p + mx2) + 2.f * mxy_xy) + my_yy) * oie;
        }
    }
}

__global__ void __launch_bounds__(256)
k_flexure_strip(const float* __restrict__ whi, const float* __restrict__ wlo, const float* __restrict__ q0,
                const uint8_t* __restrict__ mask, const float* __restrict__ D, const float* __restrict__ inv2eta,
                float* __restrict__ f, int nx, int ny, FlexCoefF c, int seg, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    const int task = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (task >= strip_tasks(nx, ny, seg)) return;   // whole warps
    flexure_strip<true>(whi, wlo, q0, mask, D, inv2eta, f, nx, ny, c, seg, task);
}

__global__ void __launch_bounds__(256)
k_flexure_strip_y(const double* __restrict__ y, const double* __restrict__ wref, const float* __restrict__ q0,
                  const uint8_t* __restrict__ mask, const float* __restrict__ D, const float* __restrict__ inv2eta,
                  float* __restrict__ f, int nx, int ny, FlexCoefF c, int seg, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    const int task = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (task >= strip_tasks(nx, ny, seg)) return;   // whole warps
    flexure_strip<false>(nullptr, nullptr, q0, mask, D, inv2eta, f, nx, ny, c, seg, task, y, wref);
}

// RK4 stage RHS from the float pair of x: stage scale sdf = (a h) spy with h
// the step size in the control block, cm the corner mean of rprev; thread 0
// forms both (the only FP64 instructions of the kernel).
__global__ void __launch_bounds__(256)
k_flexure_strip_stage(const float* __restrict__ whi, const float* __restrict__ wlo, const float* __restrict__ rprev,
                      const float* __restrict__ dxw, const float* __restrict__ q0, const uint8_t* __restrict__ mask,
                      const float* __restrict__ D, const float* __restrict__ inv2eta, float* __restrict__ f, int nx,
                      int ny, FlexCoefF c, int seg, const Ctl* __restrict__ ctl, double a, double spy,
                      const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    __shared__ float s_sc[2];
    if (threadIdx.x == 0) {
        s_sc[0] = rprev ? (float)(a * ctl->h * spy) : 0.f;
        s_sc[1] = rprev ? (float)corner_mean_of(rprev, nx, ny) : 0.f;
    }
    __syncthreads();
    const int task = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (task >= strip_tasks(nx, ny, seg)) return;   // whole warps
    flexure_strip<true, true>(whi, wlo, q0, mask, D, inv2eta, f, nx, ny, c, seg, task, nullptr, nullptr, rprev,
                              s_sc[0], s_sc[1], dxw);
}

// rows per warp task for a single domain: enough tasks to fill the GPU
static int strip_seg_single(int nx, int ny)
{
    const long long ncg = (nx + SW - 1) / SW;
    long long seg = (long long)ny * ncg / (152 * 16);
    if (seg > 32) seg = 32;
    if (seg < 8) seg = 8;
    return (int)seg;
}

__global__ void __launch_bounds__(TX* TY)
k_flexure_f32(const double* __restrict__ y, const double* __restrict__ wref, const float* __restrict__ q0,
              const uint8_t* __restrict__ mask, const float* __restrict__ D, const float* __restrict__ inv2eta,
              float* __restrict__ f, int nx, int ny, FlexCoefF c, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    flexure_f32_body<false>(y, wref, q0, mask, D, inv2eta, f, nx, ny, c, blockIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(TX* TY)
k_flexure_f32_hilo(const float* __restrict__ whi, const float* __restrict__ wlo, const float* __restrict__ q0,
                   const uint8_t* __restrict__ mask, const float* __restrict__ D, const float* __restrict__ inv2eta,
                   float* __restrict__ f, int nx, int ny, FlexCoefF c, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    flexure_f32_body<true>(nullptr, nullptr, q0, mask, D, inv2eta, f, nx, ny, c, blockIdx.x, blockIdx.y, whi, wlo);
}

template <typename T>
void launch_flexure(const double* y, const double* wref, const T* q0, const uint8_t* mask, const T* D,
                    const T* inv2eta, T* f, int nx, int ny, const FlexCoef& c, cudaStream_t s, const int* gate,
                    const float* whi, const float* wlo)
{
    dim3 b(TX, TY), g((nx + TX - 1) / TX, (ny + TY - 1) / TY);
    if (sizeof(T) == 4 && c.dxm == nullptr) {
        const FlexCoefF cf = flex_coef_f32(c);
        if (whi && !wref) {
            const int seg = strip_seg_single(nx, ny);
            const int tasks = ((nx + SW - 1) / SW) * ((ny + seg - 1) / seg);
            k_flexure_strip<<<(tasks + 7) / 8, 256, 0, s>>>(whi, wlo, (const float*)q0, mask, (const float*)D,
                                                            (const float*)inv2eta, (float*)f, nx, ny, cf, seg, gate);
            return;
        }
        // the FP64 state by column strips (the shared-memory tile form is
        // kept for FI_FLEXURE_TILES=1)
        static const bool tiles = [] {
            const char* e = getenv("FI_FLEXURE_TILES");
            return e && e[0] == '1';
        }();
        if (!tiles) {
            const int seg = strip_seg_single(nx, ny);
            const int tasks = ((nx + SW - 1) / SW) * ((ny + seg - 1) / seg);
            k_flexure_strip_y<<<(tasks + 7) / 8, 256, 0, s>>>(y, wref, (const float*)q0, mask, (const float*)D,
                                                              (const float*)inv2eta, (float*)f, nx, ny, cf, seg, gate);
            return;
        }
        k_flexure_f32<<<g, b, 0, s>>>(y, wref, (const float*)q0, mask, (const float*)D, (const float*)inv2eta,
                                      (float*)f, nx, ny, cf, gate);
        return;
    }
    k_flexure<T><<<g, b, 0, s>>>(y, wref, q0, mask, D, inv2eta, f, nx, ny, c, gate);
}

void launch_flexure_stage(const float* whi, const float* wlo, const float* rprev, const float* dxw, const float* q0,
                          const uint8_t* mask, const float* D, const float* inv2eta, float* f, int nx, int ny,
                          const FlexCoef& c, const Ctl* ctl, double a, double spy, cudaStream_t s,
                          const int* gate)
{
    const FlexCoefF cf = flex_coef_f32(c);
    const int seg = strip_seg_single(nx, ny);
    const int tasks = ((nx + SW - 1) / SW) * ((ny + seg - 1) / seg);
    k_flexure_strip_stage<<<(tasks + 7) / 8, 256, 0, s>>>(whi, wlo, rprev, dxw, q0, mask, D, inv2eta, f, nx, ny, cf,
                                                          seg, ctl, a, spy, gate);
}

// ---------------------------------------------------------------------------
// Row transforms.  A block handles RB rows; nx real samples are packed as
// h = nx/2 complex samples (z[m] = x[2m] + i x[2m+1]).
// ---------------------------------------------------------------------------
static int rows_per_block(int h)
{
    int rb = 512 / (h > 0 ? h : 1);
    if (rb < 1) rb = 1;
    if (rb > 8) rb = 8;
    return rb;
}
static int threads_for(int work)
{
    int t = 32;
    while (t < work && t < 256) t *= 2;
    return t;
}

template <typename T>
__device__ __forceinline__ void rows_fwd_body(const T* __restrict__ in, int in_pitch, int in_width, int nrows_in,
                           typename vec2<T>::type* __restrict__ S, Plan2D p, int RB, int bx, int by)
{
    typedef typename vec2<T>::type C2;
    extern __shared__ unsigned char smem_raw[];
    C2* b0 = reinterpret_cast<C2*>(smem_raw);
    C2* b1 = b0 + RB * p.h;
    const int h = p.h;
    const int j0 = bx * RB;
    const int nthr = blockDim.x;
    for (int e = threadIdx.x; e < RB * h; e += nthr) {
        const int line = e / h, m = e - line * h;
        const int j = j0 + line;
        C2 v = mk2<T>((T)0, (T)0);
        if (j < nrows_in) {
            const T* row = in + (size_t)j * in_pitch;
            const int i = 2 * m;
            if (i + 1 < in_width) {
                if ((in_pitch & 1) == 0) v = *reinterpret_cast<const C2*>(row + i);
                else v = mk2<T>(row[i], row[i + 1]);
            } else if (i < in_width) {
                v = mk2<T>(row[i], (T)0);
            }
        }
        b0[e] = v;
    }
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, p.row.d, RB, h, twp<T>(p.row), -1);
    const C2* rtw = rtwp<T>(p);
    for (int e = threadIdx.x; e < RB * (h + 1); e += nthr) {
        const int line = e / (h + 1), k = e - line * (h + 1);
        const int j = j0 + line;
        if (j >= nrows_in) continue;
        const C2 Zk = r[line * h + (k == h ? 0 : k)];
        const C2 Zc = r[line * h + (k == 0 ? 0 : h - k)];
        C2 E, O;
        E.x = (T)0.5 * (Zk.x + Zc.x);
        E.y = (T)0.5 * (Zk.y - Zc.y);
        O.x = (T)0.5 * (Zk.y + Zc.y);
        O.y = (T)-0.5 * (Zk.x - Zc.x);
        S[(size_t)j * p.sp + k] = cadd(E, cmul(__ldg(rtw + k), O));
    }
}

template <typename T>
__global__ void k_rows_fwd(const T* __restrict__ in, int in_pitch, int in_width, int nrows_in,
                           typename vec2<T>::type* __restrict__ S, Plan2D p, int RB, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    rows_fwd_body<T>(in, in_pitch, in_width, nrows_in, S, p, RB, blockIdx.x, 0);
}

template <typename T>
void launch_rows_fwd(const T* in, int in_pitch, int in_width, int nrows_in, typename vec2<T>::type* S,
                     const Plan2D& p, cudaStream_t s, const int* gate)
{
    typedef typename vec2<T>::type C2;
    const int RB = p.rb > 0 ? p.rb : rows_per_block(p.h);
    const size_t sm = 2 * (size_t)RB * p.h * sizeof(C2);
    set_smem(k_rows_fwd<T>, sm);
    const int nblk = (nrows_in + RB - 1) / RB;
    const int nt = p.rt > 0 ? p.rt : threads_for(RB * p.h / 4);
    k_rows_fwd<T><<<nblk, nt, sm, s>>>(in, in_pitch, in_width, nrows_in, S, p, RB, gate);
}

template <typename T>
__device__ __forceinline__ void rows_inv_body(const typename vec2<T>::type* __restrict__ S, int nrows, T* __restrict__ out,
                           int out_pitch, Plan2D p, int RB, T scale, int bx, int by)
{
    typedef typename vec2<T>::type C2;
    extern __shared__ unsigned char smem_raw[];
    C2* b0 = reinterpret_cast<C2*>(smem_raw);
    C2* b1 = b0 + RB * p.h;
    const int h = p.h;
    const int j0 = bx * RB;
    const int nthr = blockDim.x;
    const C2* rtw = rtwp<T>(p);
    // Z[k] = (X[k] + conj X[h-k]) + i conj(w^k) (X[k] - conj X[h-k])
    for (int e = threadIdx.x; e < RB * h; e += nthr) {
        const int line = e / h, k = e - line * h;
        const int j = j0 + line;
        C2 z = mk2<T>((T)0, (T)0);
        if (j < nrows) {
            const C2 A = S[(size_t)j * p.sp + k];
            C2 B = S[(size_t)j * p.sp + (h - k)];
            B.y = -B.y;
            const C2 sum = cadd(A, B), dif = csub(A, B);
            const C2 t = cmulc(dif, __ldg(rtw + k));
            z.x = sum.x - t.y;
            z.y = sum.y + t.x;
        }
        b0[e] = z;
    }
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, p.row.d, RB, h, twp<T>(p.row), +1);
    for (int e = threadIdx.x; e < RB * h; e += nthr) {
        const int line = e / h, m = e - line * h;
        const int j = j0 + line;
        if (j >= nrows) continue;
        C2 v = r[e];
        v.x *= scale;
        v.y *= scale;
        *reinterpret_cast<C2*>(out + (size_t)j * out_pitch + 2 * m) = v;
    }
}

template <typename T>
__global__ void k_rows_inv(const typename vec2<T>::type* __restrict__ S, int nrows, T* __restrict__ out,
                           int out_pitch, Plan2D p, int RB, T scale, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    rows_inv_body<T>(S, nrows, out, out_pitch, p, RB, scale, blockIdx.x, 0);
}

template <typename T>
void launch_rows_inv(const typename vec2<T>::type* S, T* out, const Plan2D& p, double scale, cudaStream_t s,
                     const int* gate)
{
    typedef typename vec2<T>::type C2;
    const int RB = p.rb > 0 ? p.rb : rows_per_block(p.h);
    const size_t sm = 2 * (size_t)RB * p.h * sizeof(C2);
    set_smem(k_rows_inv<T>, sm);
    const int nblk = (p.ny + RB - 1) / RB;
    const int nt = p.rt > 0 ? p.rt : threads_for(RB * p.h / 4);
    k_rows_inv<T><<<nblk, nt, sm, s>>>(S, p.ny, out, p.nx, p, RB, (T)scale, gate);
}

// ---------------------------------------------------------------------------
// Column kernels.  A block loads CB spectrum columns (all ny rows) into
// shared memory, column-major, and transforms them together.
// ---------------------------------------------------------------------------
// Columns per block: two float2 or one double2 column, i.e. 16-byte row
// segments, which keeps hundreds of blocks in flight at 512^2.
// Column c of a block lives at c * col_stride(ny) in shared memory: one
// complex element of padding per column, so the CB columns of a row segment
// (loaded and stored together) fall in different banks instead of one.
__host__ __device__ __forceinline__ int col_stride(int ny) { return ny + 1; }

template <typename T> static int cols_per_block(int ny)
{
    typedef typename vec2<T>::type C2;
    int cb = (int)(16 / sizeof(C2));
    if (cb < 1) cb = 1;
    while (cb > 1 && 2 * (size_t)cb * col_stride(ny) * sizeof(C2) > 200 * 1024) cb /= 2;
    return cb;
}

template <typename T>
__device__ __forceinline__ void load_cols(typename vec2<T>::type* b0, const typename vec2<T>::type* S, int k0,
                                          int CB, int nrows_in, const Plan2D& p)
{
    typedef typename vec2<T>::type C2;
    const int ny = p.col.d.n, ls = col_stride(ny);
    for (int e = threadIdx.x; e < CB * ny; e += blockDim.x) {
        const int c = e % CB, l = e / CB;
        const int k = k0 + c;
        C2 v = mk2<T>((T)0, (T)0);
        if (k <= p.h && l < nrows_in) v = S[(size_t)l * p.sp + k];
        b0[c * ls + l] = v;
    }
}

template <typename T>
__device__ __forceinline__ void cols_hartley_body(typename vec2<T>::type* __restrict__ S, const T* __restrict__ mA,
                               const T* __restrict__ mB, int even, Plan2D p, int CB, int bx, int by)
{
    typedef typename vec2<T>::type C2;
    extern __shared__ unsigned char smem_raw[];
    const int ny = p.col.d.n, ls = col_stride(ny);
    C2* b0 = reinterpret_cast<C2*>(smem_raw);
    C2* b1 = b0 + (size_t)CB * ls;
    const int k0 = bx * CB;
    load_cols<T>(b0, S, k0, CB, ny, p);
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, p.col.d, CB, ls, twp<T>(p.col), -1);
    const int half = ny / 2 + 1;
    for (int e = threadIdx.x; e < CB * half; e += blockDim.x) {
        const int c = e % CB, l = e / CB;
        const int k = k0 + c;
        if (k > p.h) continue;
        const int lm = (ny - l) % ny;
        C2* col = r + (size_t)c * ls;
        const size_t ia = (size_t)l * p.sp + k, ib = (size_t)lm * p.sp + k;
        const C2 Fa = col[l], Fb = col[lm];
        if (even) {
            const T ma = mA[ia], mb = mA[ib];
            C2 a = Fa, b = Fb;
            a.x *= ma; a.y *= ma;
            b.x *= mb; b.y *= mb;
            col[l] = a;
            if (lm != l) col[lm] = b;
        } else {
            // Hartley values at (k,l), (-k,-l), (-k,l), (k,-l)
            const T H_kl = Fb.x - Fa.y, H_mkml = Fb.x + Fa.y;
            const T H_mkl = Fa.x + Fb.y, H_kml = Fa.x - Fb.y;
            const T G_kl = mA[ia] * H_kl, G_kml = mA[ib] * H_kml;
            const T G_mkl = mB[ia] * H_mkl, G_mkml = mB[ib] * H_mkml;
            C2 a, b;
            a.x = (T)0.5 * (G_kml + G_mkl);
            a.y = (T)0.5 * (G_mkml - G_kl);
            b.x = (T)0.5 * (G_kl + G_mkml);
            b.y = (T)0.5 * (G_mkl - G_kml);
            col[l] = a;
            if (lm != l) col[lm] = b;
        }
    }
    __syncthreads();
    C2* other = (r == b0) ? b1 : b0;
    C2* q = block_fft<T>(r, other, p.col.d, CB, ls, twp<T>(p.col), +1);
    for (int e = threadIdx.x; e < CB * ny; e += blockDim.x) {
        const int c = e % CB, l = e / CB;
        const int k = k0 + c;
        if (k <= p.h) S[(size_t)l * p.sp + k] = q[c * ls + l];
    }
}

template <typename T>
__global__ void k_cols_hartley(typename vec2<T>::type* __restrict__ S, const T* __restrict__ mA,
                               const T* __restrict__ mB, int even, Plan2D p, int CB, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    cols_hartley_body<T>(S, mA, mB, even, p, CB, blockIdx.x, 0);
}

template <typename T>
void launch_cols_hartley(typename vec2<T>::type* S, const T* mA, const T* mB, int even, const Plan2D& p,
                         cudaStream_t s, const int* gate)
{
    typedef typename vec2<T>::type C2;
    const int CB = p.cb > 0 ? p.cb : cols_per_block<T>(p.ny);
    const size_t sm = 2 * (size_t)CB * col_stride(p.ny) * sizeof(C2);
    set_smem(k_cols_hartley<T>, sm);
    const int nblk = (p.h + 1 + CB - 1) / CB;
    const int nt = p.ct > 0 ? p.ct : threads_for(CB * p.ny / 4);
    k_cols_hartley<T><<<nblk, nt, sm, s>>>(S, mA, mB, even, p, CB, gate);
}

template <typename T>
__global__ void k_cols_conv(typename vec2<T>::type* __restrict__ S, const typename vec2<T>::type* __restrict__ K,
                            int nrows_in, const int* __restrict__ out_rows, int n_out, Plan2D p, int CB, int do_inv)
{
    typedef typename vec2<T>::type C2;
    extern __shared__ unsigned char smem_raw[];
    const int ny = p.col.d.n, ls = col_stride(ny);
    C2* b0 = reinterpret_cast<C2*>(smem_raw);
    C2* b1 = b0 + (size_t)CB * ls;
    const int k0 = blockIdx.x * CB;
    load_cols<T>(b0, S, k0, CB, nrows_in, p);
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, p.col.d, CB, ls, twp<T>(p.col), -1);
    if (!do_inv) {
        for (int e = threadIdx.x; e < CB * ny; e += blockDim.x) {
            const int c = e % CB, l = e / CB;
            const int k = k0 + c;
            if (k <= p.h) S[(size_t)l * p.sp + k] = r[c * ls + l];
        }
        return;
    }
    for (int e = threadIdx.x; e < CB * ny; e += blockDim.x) {
        const int c = e % CB, l = e / CB;
        const int k = k0 + c;
        if (k > p.h) continue;
        r[c * ls + l] = cmul(r[c * ls + l], K[(size_t)l * p.sp + k]);
    }
    __syncthreads();
    C2* other = (r == b0) ? b1 : b0;
    C2* q = block_fft<T>(r, other, p.col.d, CB, ls, twp<T>(p.col), +1);
    for (int e = threadIdx.x; e < CB * n_out; e += blockDim.x) {
        const int c = e % CB, o = e / CB;
        const int k = k0 + c;
        if (k <= p.h) S[(size_t)o * p.sp + k] = q[c * ls + out_rows[o]];
    }
}

template <typename T>
void launch_cols_conv(typename vec2<T>::type* S, const typename vec2<T>::type* K, int nrows_in, const int* out_rows,
                      int n_out, const Plan2D& p, cudaStream_t s)
{
    typedef typename vec2<T>::type C2;
    const int CB = p.cb > 0 ? p.cb : cols_per_block<T>(p.ny);
    const size_t sm = 2 * (size_t)CB * col_stride(p.ny) * sizeof(C2);
    set_smem(k_cols_conv<T>, sm);
    const int nblk = (p.h + 1 + CB - 1) / CB;
    const int nt = p.ct > 0 ? p.ct : threads_for(CB * p.ny / 4);
    k_cols_conv<T><<<nblk, nt, sm, s>>>(S, K, nrows_in, out_rows, n_out, p, CB, 1);
}

template <typename T>
void launch_cols_fwd(typename vec2<T>::type* S, int nrows_in, const Plan2D& p, cudaStream_t s)
{
    typedef typename vec2<T>::type C2;
    const int CB = p.cb > 0 ? p.cb : cols_per_block<T>(p.ny);
    const size_t sm = 2 * (size_t)CB * col_stride(p.ny) * sizeof(C2);
    set_smem(k_cols_conv<T>, sm);
    const int nblk = (p.h + 1 + CB - 1) / CB;
    k_cols_conv<T><<<nblk, threads_for(CB * p.ny / 4), sm, s>>>(S, nullptr, nrows_in, nullptr, 0, p, CB, 0);
}

// Inverse rows of the compacted convolution spectrum.  Rows 0..ny-1 are the
// cropped output rows; rows ny and ny+1 are the linear-lag rows 0 and
// 2*ny-2 that hold the corner values of apply_zerobc_at_corners_dp.
template <typename T>
__global__ void k_conv_rows_inv(const typename vec2<T>::type* __restrict__ S, int n_out, double* __restrict__ out,
                                int nx, int ny, int i_off, double* __restrict__ corners, int col1, Plan2D p,
                                int RB, T scale)
{
    typedef typename vec2<T>::type C2;
    extern __shared__ unsigned char smem_raw[];
    C2* b0 = reinterpret_cast<C2*>(smem_raw);
    C2* b1 = b0 + RB * p.h;
    const int h = p.h;
    const int j0 = blockIdx.x * RB;
    const int nthr = blockDim.x;
    const C2* rtw = rtwp<T>(p);
    for (int e = threadIdx.x; e < RB * h; e += nthr) {
        const int line = e / h, k = e - line * h;
        const int j = j0 + line;
        C2 z = mk2<T>((T)0, (T)0);
        if (j < n_out) {
            const C2 A = S[(size_t)j * p.sp + k];
            C2 B = S[(size_t)j * p.sp + (h - k)];
            B.y = -B.y;
            const C2 sum = cadd(A, B), dif = csub(A, B);
            const C2 t = cmulc(dif, __ldg(rtw + k));
            z.x = sum.x - t.y;
            z.y = sum.y + t.x;
        }
        b0[e] = z;
    }
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, p.row.d, RB, h, twp<T>(p.row), +1);
    const T* rr = reinterpret_cast<const T*>(r);
    for (int e = threadIdx.x; e < RB * nx; e += nthr) {
        const int line = e / nx, i = e - line * nx;
        const int j = j0 + line;
        if (j < ny) out[(size_t)j * nx + i] = (double)(rr[(size_t)line * 2 * h + i_off + i] * scale);
    }
    if (threadIdx.x == 0) {
        for (int line = 0; line < RB; ++line) {
            const int j = j0 + line;
            const T* row = rr + (size_t)line * 2 * h;
            if (j == ny) {            // linear lag row 0
                corners[0] = (double)(row[0] * scale);
                corners[3] = (double)(row[col1] * scale);
            } else if (j == ny + 1) { // linear lag row 2*ny-2
                corners[2] = (double)(row[0] * scale);
                corners[1] = (double)(row[col1] * scale);
            }
        }
    }
}

template <typename T>
void launch_conv_rows_inv(const typename vec2<T>::type* S, int n_out, double* out, int nx, int ny, int i_off,
                          double* corners, int /*corner_row0*/, int /*corner_row1*/, int corner_col1,
                          const Plan2D& p, double scale, cudaStream_t s)
{
    typedef typename vec2<T>::type C2;
    const int RB = p.rb > 0 ? p.rb : rows_per_block(p.h);
    const size_t sm = 2 * (size_t)RB * p.h * sizeof(C2);
    set_smem(k_conv_rows_inv<T>, sm);
    const int nblk = (n_out + RB - 1) / RB;
    const int nt = p.rt > 0 ? p.rt : threads_for(RB * p.h / 4);
    k_conv_rows_inv<T><<<nblk, nt, sm, s>>>(S, n_out, out, nx, ny, i_off, corners, corner_col1, p, RB, (T)scale);
}

// ---------------------------------------------------------------------------
// Batched launches: the same bodies over every member of an ensemble.  A
// member whose attempt needs no new RHS (need_rhs == 0) returns at once.
// ---------------------------------------------------------------------------
int rhs_rows_per_block(int h) { return rows_per_block(h); }
int rhs_threads_for(int work) { return threads_for(work); }
template <typename T> int rhs_cols_per_block(int ny) { return cols_per_block<T>(ny); }
template int rhs_cols_per_block<float>(int);
template int rhs_cols_per_block<double>(int);

template <typename T>
__global__ void __launch_bounds__(256) k_b_flexure(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { return true; }, [&](int m, int local) {   // the list holds the members with work
        const BMember& b = M[m];
        const int bx = local % b.fgx, by = local / b.fgx;
        if constexpr (sizeof(T) == 4) {
            // mixed members have uniform spacing and carry now%w as a float
            // pair: column strips, 8 warp tasks per virtual block
            const int task = local * 8 + (int)threadIdx.y;   // 32 x 8 block: warp = threadIdx.y
            if (task < strip_tasks(b.p.nx, b.p.ny, b.fseg))
                flexure_strip<true>(b.d.whi, b.d.wlo, (const float*)b.q0, b.mask, (const float*)b.D,
                              (const float*)b.inv2eta, (float*)b.f, b.p.nx, b.p.ny, b.fcf, b.fseg, task);
        } else {
            flexure_body<T>(b.y, nullptr, (const T*)b.q0, b.mask, (const T*)b.D, (const T*)b.inv2eta, (T*)b.f,
                            b.p.nx, b.p.ny, b.fc, bx, by);
        }
        __syncthreads();   // the next virtual block reuses the shared tiles
    });
}

template <typename T>
__global__ void k_b_rows_fwd(const BMember* __restrict__ M, BList L)
{
    typedef typename vec2<T>::type C2;
    batch_walk(L, [&](int m) { return true; }, [&](int m, int local) {   // the list holds the members with work
        const BMember& b = M[m];
        rows_fwd_body<T>((const T*)b.f, b.p.nx, b.p.nx, b.p.ny, (C2*)b.S, b.p, b.RB, local, 0);
        __syncthreads();
    });
}

template <typename T>
__global__ void k_b_cols_hartley(const BMember* __restrict__ M, BList L)
{
    typedef typename vec2<T>::type C2;
    batch_walk(L, [&](int m) { return true; }, [&](int m, int local) {   // the list holds the members with work
        const BMember& b = M[m];
        cols_hartley_body<T>((C2*)b.S, (const T*)b.mA, (const T*)b.mB, b.even, b.p, b.CB, local, 0);
        __syncthreads();
    });
}

template <typename T>
__global__ void k_b_rows_inv(const BMember* __restrict__ M, BList L, int stage)
{
    typedef typename vec2<T>::type C2;
    batch_walk(L, [&](int m) { return true; }, [&](int m, int local) {
        const BMember& b = M[m];
        T scale;   // 1/(nx*ny*1.), converted on the host
        if constexpr (sizeof(T) == 4) scale = b.norm_scale_f;
        else scale = b.norm_scale;
        rows_inv_body<T>((const C2*)b.S, b.p.ny, (T*)b.raw7[stage], b.p.nx, b.p, b.RB, scale, local, 0);
        __syncthreads();
    });
}

template <typename T> void batch_grids(size_t rows_smem, size_t cols_smem, int rows_threads, int cols_threads,
                                       int* g_flex, int* g_rows, int* g_cols, int* g_red)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    auto resident = [&](auto kern, int threads, size_t smem) {
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem) != cudaSuccess || per < 1) per = 1;
        return per * nsm;
    };
    *g_flex = resident(k_b_flexure<T>, TX * TY, 0);
    *g_rows = resident(k_b_rows_fwd<T>, rows_threads, rows_smem);
    const int gi = resident(k_b_rows_inv<T>, rows_threads, rows_smem);
    if (gi < *g_rows) *g_rows = gi;
    *g_cols = resident(k_b_cols_hartley<T>, cols_threads, cols_smem);
    *g_red = batch_red_resident<T>() * nsm;
}

template <typename T> void batch_flexure(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    // 256 threads: the tile body reads them as TX x TY, the strip body as 8 warps
    k_b_flexure<T><<<nblk, dim3(TX, TY), 0, s>>>(M, L);
}
int batch_flexure_blocks(int nx, int ny, int seg) { return (((nx + SW - 1) / SW) * ((ny + seg - 1) / seg) + 7) / 8; }
template <typename T>
void batch_rows_fwd(const BMember* M, BList L, int nblk, int threads, size_t smem, cudaStream_t s)
{
    set_smem(k_b_rows_fwd<T>, smem);
    k_b_rows_fwd<T><<<nblk, threads, smem, s>>>(M, L);
}
template <typename T>
void batch_cols_hartley(const BMember* M, BList L, int nblk, int threads, size_t smem, cudaStream_t s)
{
    set_smem(k_b_cols_hartley<T>, smem);
    k_b_cols_hartley<T><<<nblk, threads, smem, s>>>(M, L);
}
template <typename T>
void batch_rows_inv(const BMember* M, BList L, int nblk, int threads, size_t smem, cudaStream_t s, int stage)
{
    set_smem(k_b_rows_inv<T>, smem);
    k_b_rows_inv<T><<<nblk, threads, smem, s>>>(M, L, stage);
}

// True stages: the RHS at stage state y (stage 0: x, 1-5: the stage buffer,
// 6: x2) with the mantle term at that state: mixed members by column strips
// over the float pair of the stage state (stage 0: of x) and its dxw, FP64
// members (and mixed ones without the pairs) by shared-memory tiles.
template <typename T>
__global__ void __launch_bounds__(256) k_b_flexure_y(const BMember* __restrict__ M, BList L, int stage)
{
    batch_walk(L, [&](int m) { return true; }, [&](int m, int local) {
        const BMember& b = M[m];
        const int bx = local % b.fgx, by = local / b.fgx;
        const double* y = stage == 0 ? b.d.x : (stage == 6 ? b.d.ts_x2 : b.yst);
        if constexpr (sizeof(T) == 4) {
            if (b.yhi) {
                const int task = local * 8 + (int)threadIdx.y;   // 32 x 8 block: warp = threadIdx.y
                if (task < strip_tasks(b.p.nx, b.p.ny, b.fseg)) {
                    const bool s0 = stage == 0;
                    flexure_strip<true, true>(s0 ? b.xhi : b.yhi, s0 ? b.xlo : b.ylo, (const float*)b.q0, b.mask,
                                              (const float*)b.D, (const float*)b.inv2eta, (float*)b.f, b.p.nx,
                                              b.p.ny, b.fcf, b.fseg, task, nullptr, nullptr, nullptr, 0.f, 0.f,
                                              s0 ? b.xdw : b.ydw);
                }
            } else {
                flexure_f32_body<false>(y, b.wref, (const float*)b.q0, b.mask, (const float*)b.D,
                                        (const float*)b.inv2eta, (float*)b.f, b.p.nx, b.p.ny, b.fcf, bx, by);
            }
        } else {
            flexure_body<T>(y, b.wref, (const T*)b.q0, b.mask, (const T*)b.D, (const T*)b.inv2eta, (T*)b.f, b.p.nx,
                            b.p.ny, b.fc, bx, by);
        }
        __syncthreads();
    });
}
template <typename T> void batch_flexure_y(const BMember* M, BList L, int nblk, int stage, cudaStream_t s)
{
    k_b_flexure_y<T><<<nblk, dim3(TX, TY), 0, s>>>(M, L, stage);
}

template <typename T> void batch_prepare(size_t rows_smem, size_t cols_smem)
{
    set_smem(k_b_rows_fwd<T>, rows_smem);
    set_smem(k_b_rows_inv<T>, rows_smem);
    set_smem(k_b_cols_hartley<T>, cols_smem);
}

#define FI_BATCH_INST(T)                                                                                   \
    template void batch_prepare<T>(size_t, size_t);                                                        \
    template void batch_grids<T>(size_t, size_t, int, int, int*, int*, int*, int*);                        \
    template void batch_flexure<T>(const BMember*, BList, int, cudaStream_t);                    \
    template void batch_rows_fwd<T>(const BMember*, BList, int, int, size_t, cudaStream_t);      \
    template void batch_cols_hartley<T>(const BMember*, BList, int, int, size_t, cudaStream_t);  \
    template void batch_rows_inv<T>(const BMember*, BList, int, int, size_t, cudaStream_t, int);      \
    template void batch_flexure_y<T>(const BMember*, BList, int, int, cudaStream_t);
FI_BATCH_INST(double)
FI_BATCH_INST(float)

#define FI_INST(T)                                                                                            \
    template void launch_flexure<T>(const double*, const double*, const T*, const uint8_t*, const T*, const T*, \
                                    T*, int, int, const FlexCoef&, cudaStream_t, const int*, const float*,    \
                                    const float*);                                                            \
    template void launch_rows_fwd<T>(const T*, int, int, int, vec2<T>::type*, const Plan2D&, cudaStream_t,    \
                                     const int*);                                                             \
    template void launch_cols_hartley<T>(vec2<T>::type*, const T*, const T*, int, const Plan2D&, cudaStream_t, \
                                         const int*);                                                         \
    template void launch_rows_inv<T>(const vec2<T>::type*, T*, const Plan2D&, double, cudaStream_t, const int*); \
    template void launch_cols_conv<T>(vec2<T>::type*, const vec2<T>::type*, int, const int*, int, const Plan2D&, \
                                      cudaStream_t);                                                          \
    template void launch_cols_fwd<T>(vec2<T>::type*, int, const Plan2D&, cudaStream_t);                       \
    template void launch_conv_rows_inv<T>(const vec2<T>::type*, int, double*, int, int, int, double*, int, int,  \
                                          int, const Plan2D&, double, cudaStream_t);

FI_INST(double)
FI_INST(float)

}  // namespace fi
