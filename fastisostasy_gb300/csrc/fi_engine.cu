// fi_engine.cu — persistent cooperative RK4 step engine.
//
// One cooperative launch integrates all RK4 steps of an isos_update
// (step_rk4 with true stages, src/integrators.f90:42-77, evaluating
// calc_lvelva, src/lv_elva.f90:31-126, at every stage state).  The grid
// walks through phases separated by grid-wide barriers:
//
//   A  stencil + row real-FFT   (work item = 2 grid rows, full width)
//   B  column FFT, multiply by 1/(kappa R) in the Hartley basis, inverse
//   C  inverse row real-FFT -> raw_s (stage output before corner BC / sec_per_year)
//   D  x += h/6 (k1 + 2 k2 + 2 k3 + k4), w = x
//
// Stage states y_s = x + a_s h k_{s-1} are never stored: phase A rebuilds the
// differences it needs from x and raw_{s-1} (the corner mean of raw cancels
// in every difference and enters only the mantle term).  In the mixed form x
// also lives as a float hi/lo pair (x = hi + lo), so the forward differences
// dX = (hi[i+1]-hi[i]) + (lo[i+1]-lo[i]) + s (raw[i+1]-raw[i]) are formed in
// float without losing the curvature of a large smooth field; the only
// double arithmetic left is the state update of phase D.
#include <cooperative_groups.h>

#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "fi_engine.h"
#include "fi_fft.cuh"

namespace cg = cooperative_groups;

namespace fi {

template <typename T> __device__ __forceinline__ const typename vec2<T>::type* etw(const FftLen& L);
template <> __device__ __forceinline__ const double2* etw<double>(const FftLen& L) { return L.tw64; }
template <> __device__ __forceinline__ const float2* etw<float>(const FftLen& L) { return L.tw32; }
template <typename T> __device__ __forceinline__ const typename vec2<T>::type* ertw(const Plan2D& p);
template <> __device__ __forceinline__ const double2* ertw<double>(const Plan2D& p) { return p.rtw64; }
template <> __device__ __forceinline__ const float2* ertw<float>(const Plan2D& p) { return p.rtw32; }

constexpr int RA = 2;   // rows per phase-A item (must be even: see the y-boundary stencils)
constexpr int RC = 2;   // rows per phase-C item

// stage coefficients of RK4: y_s = x + a_s h k_{s-1}
__constant__ double c_rk4_a[4] = {0.0, 0.5, 0.5, 1.0};

// Shared-memory plan of phase A, in rows of nx field values (T):
//   R1 (18 rows): prefetched state rows, later Wx (6) + Mxx, Myy, Mxy (4 each)
//   R2 (17 rows): dX (6), dY (5), load term P (2), Mxyx (4)
//   R3 (10 rows): D (4), q0 (2), 1/(2 eta) (2), w_ref (2; hi/lo halves in the mixed form)
//   mask (2 rows of bytes), FFT ping-pong buffers (2 x RA rows of complex half-rows)
constexpr int A_R1 = 18, A_R2 = 17, A_R3 = 10;
template <typename T> struct PhaseAMem {
    static size_t bytes(int nx, int h)
    {
        typedef typename vec2<T>::type C2;
        size_t b = (size_t)(A_R1 + A_R2 + A_R3) * nx * sizeof(T);
        b += ((size_t)2 * nx + 15) / 16 * 16;
        b += 2 * (size_t)RA * h * sizeof(C2);
        return b;
    }
};

template <typename T> size_t engine_smem_bytes(const Plan2D& p, int CB)
{
    typedef typename vec2<T>::type C2;
    size_t a = PhaseAMem<T>::bytes(p.nx, p.h);
    size_t b = 2 * (size_t)CB * p.ny * sizeof(C2);
    size_t c = 2 * (size_t)RC * p.h * sizeof(C2);
    size_t m = a > b ? a : b;
    return (m > c ? m : c) + 64;
}

template <typename T> __device__ __forceinline__ double corner_mean_dev(const T* a, int nx, int ny)
{
    return corner_mean_of(a, nx, ny);
}

// ---------------------------------------------------------------------------
// Phase A: one item = output rows j0, j0+1 (full width).  Every global row the
// item needs is first copied into shared memory with vector loads (all in
// flight together); the stencil then runs from shared memory only.
// ---------------------------------------------------------------------------
template <typename V, bool RO, typename T>
__device__ __forceinline__ void rows_to_smem(T* dst, const T* __restrict__ src, int nrows, int gj0, int nx, int ny)
{
    // nrows rows starting at global row gj0 (zeros outside the domain); V is
    // a 16-byte vector of T.  RO: the source is read-only for the whole
    // kernel (non-coherent cache path allowed); data written by other blocks
    // during the kernel is read with coherent loads.
    constexpr int W = sizeof(V) / sizeof(T);
    const int nv = nx / W;
    const int tot = nrows * nv;
    V* d = reinterpret_cast<V*>(dst);
    for (int e0 = threadIdx.x; e0 < tot; e0 += 4 * blockDim.x) {
        V v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < tot) {
                const int r = e / nv, c = e - r * nv;
                const int gj = gj0 + r;
                if (gj >= 0 && gj < ny) {
                    const V* ps = reinterpret_cast<const V*>(src + (size_t)gj * nx) + c;
                    v[u] = RO ? __ldg(ps) : *ps;
                }
                else v[u] = V{};
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < tot) d[e] = v[u];
        }
    }
}

template <typename T>
__device__ void phase_a(const EngineArgs& g, int j0, int stage, double h, unsigned char* smem)
{
    typedef typename vec2<T>::type C2;
    typedef typename std::conditional<std::is_same<T, float>::value, float4, double2>::type V;
    const int nx = g.p.nx, ny = g.p.ny, hh = g.p.h;
    const int tid = threadIdx.x, nt = blockDim.x;
    T* R1 = reinterpret_cast<T*>(smem);
    T* R2 = R1 + (size_t)A_R1 * nx;
    T* R3 = R2 + (size_t)A_R2 * nx;
    uint8_t* MK = reinterpret_cast<uint8_t*>(R3 + (size_t)A_R3 * nx);
    C2* b0 = reinterpret_cast<C2*>(MK + ((size_t)2 * nx + 15) / 16 * 16);
    C2* b1 = b0 + (size_t)RA * hh;
    // R1 roles
    T* XA = R1;                    // 6 rows: xhi (mixed) | x (plain)
    T* XB = R1 + 6 * (size_t)nx;   // 6 rows: xlo (mixed) | raw_prev (plain)
    T* XC = R1 + 12 * (size_t)nx;  // 6 rows: raw_prev (mixed) | y (plain)
    T* Wx = R1;                    // 6 rows   (after level 0)
    T* Mxx = R1 + 6 * (size_t)nx;  // 4 rows
    T* Myy = R1 + 10 * (size_t)nx; // 4 rows
    T* Mxy = R1 + 14 * (size_t)nx; // 4 rows
    // R2 roles
    T* dX = R2;
    T* dY = R2 + 6 * (size_t)nx;
    T* P = R2 + 11 * (size_t)nx;
    T* Mxyx = R2 + 13 * (size_t)nx;
    // R3 roles
    T* Dr = R3;
    T* Q0 = R3 + 4 * (size_t)nx;
    T* I2E = R3 + 6 * (size_t)nx;

    const T* rprev = stage > 0 ? (const T*)g.raw[stage - 1] : nullptr;
    __shared__ double s_sc[2];
    if (tid == 0) {
        // y = x + a h spy (raw - cm): the scale s and the corner mean cm
        s_sc[0] = stage > 0 ? c_rk4_a[stage] * h * g.spy : 0.0;
        s_sc[1] = stage > 0 ? corner_mean_of(rprev, nx, ny) : 0.0;
    }
    // ---- prefetch
    if constexpr (std::is_same<T, float>::value) {
        rows_to_smem<V, false>(XA, g.xhi, 6, j0 - 2, nx, ny);
        rows_to_smem<V, false>(XB, g.xlo, 6, j0 - 2, nx, ny);
        if (rprev) rows_to_smem<V, false>(XC, rprev, 6, j0 - 2, nx, ny);
    } else {
        rows_to_smem<V, false>(XA, g.x, 6, j0 - 2, nx, ny);
        if (rprev) rows_to_smem<V, false>(XB, rprev, 6, j0 - 2, nx, ny);
    }
    rows_to_smem<V, true>(Dr, g.D_T<T>(), 4, j0 - 1, nx, ny);
    rows_to_smem<V, true>(Q0, g.q0_T<T>(), 2, j0, nx, ny);
    rows_to_smem<V, true>(I2E, g.inv2eta_T<T>(), 2, j0, nx, ny);
    for (int e = tid; e < 2 * nx; e += nt) {
        const int o = e / nx, i = e - o * nx;
        MK[e] = (j0 + o < ny) ? g.mask[(size_t)(j0 + o) * nx + i] : 0;
    }
    __syncthreads();
    const double sd = s_sc[0], cmd = s_sc[1];
    // plain form: materialise the stage state y = x + s (raw - cm) in double
    if constexpr (!std::is_same<T, float>::value) {
        for (int e = tid; e < 6 * nx; e += nt) {
            double v = XA[e];
            if (rprev) v += sd * ((double)XB[e] - cmd);
            XC[e] = v;
        }
        __syncthreads();
    }
    // ---- level 0: forward differences and the load term
    const float sf = (float)sd;
    for (int e = tid; e < 6 * nx; e += nt) {
        const int r = e / nx, i = e - r * nx;
        const int gj = j0 - 2 + r;
        if (gj < 0 || gj >= ny) continue;
        if (i < nx - 1) {
            if constexpr (std::is_same<T, float>::value) {
                float v = (XA[e + 1] - XA[e]) + (XB[e + 1] - XB[e]);
                if (rprev) v += sf * (XC[e + 1] - XC[e]);
                dX[e] = v;
            } else {
                dX[e] = XC[e + 1] - XC[e];
            }
        }
        if (r < 5 && gj + 1 < ny) {
            if constexpr (std::is_same<T, float>::value) {
                float v = (XA[e + nx] - XA[e]) + (XB[e + nx] - XB[e]);
                if (rprev) v += sf * (XC[e + nx] - XC[e]);
                dY[e] = v;
            } else {
                dY[e] = XC[e + nx] - XC[e];
            }
        }
    }
    for (int e = tid; e < 2 * nx; e += nt) {
        const int o = e / nx, i = e - o * nx;
        const int gj = j0 + o;
        T p = (T)0;
        if (gj < ny && MK[e]) {
            const size_t c = (size_t)gj * nx + i;
            const int eo = (o + 2) * nx + i;   // row of the output cell in the 6-row prefetch
            // q0 + (-g rho_m) (y - w_ref) at the stage state
            if constexpr (std::is_same<T, float>::value) {
                float dy = (XA[eo] - g.wrefhi[c]) + (XB[eo] - g.wreflo[c]);
                if (rprev) dy += sf * (XC[eo] - (float)cmd);
                p = Q0[e] + (float)g.fc.coef_mantle * dy;
            } else {
                p = Q0[e] + g.fc.coef_mantle * (XC[eo] - g.wref[c]);
            }
        }
        P[e] = p;
    }
    __syncthreads();
    const T inv_dx = (T)g.fc.inv_dx, inv_2dx = (T)g.fc.inv_2dx, inv_dx2 = (T)g.fc.inv_dx2;
    const T inv_dy = (T)g.fc.inv_dy, inv_2dy = (T)g.fc.inv_2dy, inv_dy2 = (T)g.fc.inv_dy2;
    for (int e = tid; e < 6 * nx; e += nt) {
        const int r = e / nx, i = e - r * nx;
        const int gj = j0 - 2 + r;
        if (gj < 0 || gj >= ny) continue;
        const T* d = dX + (size_t)r * nx;
        T v;
        if (i == 0) v = d[0] * inv_dx;
        else if (i == nx - 1) v = d[nx - 2] * inv_dx;
        else v = (d[i] + d[i - 1]) * inv_2dx;
        Wx[e] = v;
    }
    __syncthreads();
    // ---- level 1: moments on rows j0-1 .. j0+2 (prefetch rows 1..4)
    const T nu = (T)g.fc.nu, omn = (T)g.fc.one_minus_nu;
    for (int e = tid; e < 4 * nx; e += nt) {
        const int m = e / nx, i = e - m * nx;
        const int r = m + 1;
        const int gj = j0 - 2 + r;
        if (gj < 0 || gj >= ny) continue;
        const int ri = r * nx + i;
        T wxy, wxx, wyy;
        if (gj == 0) wxy = (Wx[ri + nx] - Wx[ri]) * inv_dy;
        else if (gj == ny - 1) wxy = (Wx[ri] - Wx[ri - nx]) * inv_dy;
        else wxy = (Wx[ri + nx] - Wx[ri - nx]) * inv_2dy;
        const T* d = dX + (size_t)r * nx;
        if (i == 0) wxx = (d[1] - d[0]) * inv_dx2;
        else if (i == nx - 1) wxx = (d[nx - 2] - d[nx - 3]) * inv_dx2;
        else wxx = (d[i] - d[i - 1]) * inv_dx2;
        if (gj == 0) wyy = (dY[ri + nx] - dY[ri]) * inv_dy2;
        else if (gj == ny - 1) wyy = (dY[ri - nx] - dY[ri - 2 * nx]) * inv_dy2;
        else wyy = (dY[ri] - dY[ri - nx]) * inv_dy2;
        const T Dl = Dr[e];
        Mxx[e] = -Dl * (wxx + nu * wyy);
        Myy[e] = -Dl * (wyy + nu * wxx);
        Mxy[e] = (-Dl * omn) * wxy;
    }
    __syncthreads();
    for (int e = tid; e < 4 * nx; e += nt) {
        const int m = e / nx, i = e - m * nx;
        const int gj = j0 - 1 + m;
        if (gj < 0 || gj >= ny) continue;
        const T* M = Mxy + (size_t)m * nx;
        T v;
        if (i == 0) v = (M[1] - M[0]) * inv_dx;
        else if (i == nx - 1) v = (M[nx - 1] - M[nx - 2]) * inv_dx;
        else v = (M[i + 1] - M[i - 1]) * inv_2dx;
        Mxyx[e] = v;
    }
    __syncthreads();
    // ---- level 2 on the two output rows -> packed into the FFT buffer
    for (int e = tid; e < 2 * nx; e += nt) {
        const int o = e / nx, i = e - o * nx;
        const int gj = j0 + o;
        T fv = (T)0;
        if (gj < ny) {
            const int mi = (o + 1) * nx + i;
            T mxy_xy, mx_xx, my_yy;
            if (gj == 0) mxy_xy = (Mxyx[mi + nx] - Mxyx[mi]) * inv_dy;
            else if (gj == ny - 1) mxy_xy = (Mxyx[mi] - Mxyx[mi - nx]) * inv_dy;
            else mxy_xy = (Mxyx[mi + nx] - Mxyx[mi - nx]) * inv_2dy;
            const T* M = Mxx + (size_t)(o + 1) * nx;
            if (i == 0) mx_xx = ((M[2] - (T)2 * M[1]) + M[0]) * inv_dx2;
            else if (i == nx - 1) mx_xx = ((M[nx - 1] - (T)2 * M[nx - 2]) + M[nx - 3]) * inv_dx2;
            else mx_xx = ((M[i + 1] - (T)2 * M[i]) + M[i - 1]) * inv_dx2;
            if (gj == 0) my_yy = ((Myy[mi + 2 * nx] - (T)2 * Myy[mi + nx]) + Myy[mi]) * inv_dy2;
            else if (gj == ny - 1) my_yy = ((Myy[mi] - (T)2 * Myy[mi - nx]) + Myy[mi - 2 * nx]) * inv_dy2;
            else my_yy = ((Myy[mi + nx] - (T)2 * Myy[mi]) + Myy[mi - nx]) * inv_dy2;
            fv = (((P[e] + mx_xx) + (T)2 * mxy_xy) + my_yy) * I2E[e];
        }
        reinterpret_cast<T*>(b0)[e] = fv;   // row o at b0 + o*hh complex = o*nx reals
    }
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, g.p.row.d, RA, hh, etw<T>(g.p.row), -1);
    const C2* rtw = ertw<T>(g.p);
    C2* S = (C2*)g.S;
    for (int e = tid; e < RA * (hh + 1); e += nt) {
        const int o = e / (hh + 1), k = e - o * (hh + 1);
        const int gj = j0 + o;
        if (gj >= ny) continue;
        const C2 Zk = r[o * hh + (k == hh ? 0 : k)];
        const C2 Zc = r[o * hh + (k == 0 ? 0 : hh - k)];
        C2 E, O;
        E.x = (T)0.5 * (Zk.x + Zc.x);
        E.y = (T)0.5 * (Zk.y - Zc.y);
        O.x = (T)0.5 * (Zk.y + Zc.y);
        O.y = (T)-0.5 * (Zk.x - Zc.x);
        S[(size_t)gj * g.p.sp + k] = cadd(E, cmul(__ldg(rtw + k), O));
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Phase B: CB spectrum columns: forward column FFT, Hartley-basis multiply,
// inverse column FFT.
// ---------------------------------------------------------------------------
template <typename T>
__device__ void phase_b(const EngineArgs& g, int k0, int CB, unsigned char* smem)
{
    typedef typename vec2<T>::type C2;
    const int ny = g.p.ny;
    C2* b0 = reinterpret_cast<C2*>(smem);
    C2* b1 = b0 + (size_t)CB * ny;
    C2* S = (C2*)g.S;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e0 = tid; e0 < CB * ny; e0 += 4 * nt) {
        C2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = e0 + u * nt;
            const int c = e % CB, l = e / CB;
            const int k = k0 + c;
            v[u] = (e < CB * ny && k <= g.p.h) ? S[(size_t)l * g.p.sp + k] : mk2<T>((T)0, (T)0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = e0 + u * nt;
            if (e < CB * ny) b0[(e % CB) * ny + e / CB] = v[u];
        }
    }
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, g.p.col.d, CB, ny, etw<T>(g.p.col), -1);
    const T* mA = g.mA_T<T>();
    const T* mB = g.mB_T<T>();
    const int half = ny / 2 + 1;
    for (int e = tid; e < CB * half; e += nt) {
        const int c = e % CB, l = e / CB;
        const int k = k0 + c;
        if (k > g.p.h) continue;
        const int lm = (ny - l) % ny;
        C2* col = r + (size_t)c * ny;
        const size_t ia = (size_t)l * g.p.sp + k, ib = (size_t)lm * g.p.sp + k;
        const C2 Fa = col[l], Fb = col[lm];
        if (g.even) {
            const T ma = mA[ia], mb = mA[ib];
            C2 a = Fa, b = Fb;
            a.x *= ma; a.y *= ma;
            b.x *= mb; b.y *= mb;
            col[l] = a;
            if (lm != l) col[lm] = b;
        } else {
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
    C2* q = block_fft<T>(r, other, g.p.col.d, CB, ny, etw<T>(g.p.col), +1);
    for (int e = tid; e < CB * ny; e += nt) {
        const int c = e % CB, l = e / CB;
        const int k = k0 + c;
        if (k <= g.p.h) S[(size_t)l * g.p.sp + k] = q[c * ny + l];
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Phase C: inverse row real-FFT of rows j0 .. j0+RC-1 -> raw (scaled 1/(nx ny)).
// ---------------------------------------------------------------------------
template <typename T>
__device__ void phase_c(const EngineArgs& g, int j0, T* out, unsigned char* smem)
{
    typedef typename vec2<T>::type C2;
    const int hh = g.p.h, ny = g.p.ny, nx = g.p.nx;
    C2* b0 = reinterpret_cast<C2*>(smem);
    C2* b1 = b0 + (size_t)RC * hh;
    const C2* S = (const C2*)g.S;
    const C2* rtw = ertw<T>(g.p);
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < RC * hh; e += nt) {
        const int o = e / hh, k = e - o * hh;
        const int j = j0 + o;
        C2 z = mk2<T>((T)0, (T)0);
        if (j < ny) {
            const C2 A = S[(size_t)j * g.p.sp + k];
            C2 B = S[(size_t)j * g.p.sp + (hh - k)];
            B.y = -B.y;
            const C2 sum = cadd(A, B), dif = csub(A, B);
            const C2 t = cmulc(dif, __ldg(rtw + k));
            z.x = sum.x - t.y;
            z.y = sum.y + t.x;
        }
        b0[e] = z;
    }
    __syncthreads();
    C2* r = block_fft<T>(b0, b1, g.p.row.d, RC, hh, etw<T>(g.p.row), +1);
    const T scale = (T)g.norm_scale;
    for (int e = tid; e < RC * hh; e += nt) {
        const int o = e / hh, m = e - o * hh;
        const int j = j0 + o;
        if (j >= ny) continue;
        C2 v = r[e];
        v.x *= scale;
        v.y *= scale;
        *reinterpret_cast<C2*>(out + (size_t)j * nx + 2 * m) = v;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// MINB blocks per SM: 2 caps the registers at 128 per thread
template <typename T, int MINB>
__global__ void __launch_bounds__(256, MINB) k_engine_rk4(EngineArgs g)
{
    extern __shared__ __align__(16) unsigned char smem[];
    cg::grid_group grid = cg::this_grid();
    const int nx = g.p.nx, ny = g.p.ny;
    const size_t n = (size_t)nx * ny;
    const int na = (ny + RA - 1) / RA, nb = (g.p.h + 1 + g.CB - 1) / g.CB, nc = (ny + RC - 1) / RC;
    Ctl* ctl = g.ctl;
    __shared__ double s_h;
    const bool tr = g.trace && blockIdx.x == 0 && threadIdx.x == 0;
    int tk = 0;
#define TRACE() do { if (tr && step == 0 && tk < 64) g.trace[tk++] = gtimer(); } while (0)
    for (int step = 0; step < g.nsteps; ++step) {
        TRACE();
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            // step_rk4: h = min(dt, tf - t) (src/integrators.f90:62-63)
            if (ctl->status == ST_OK && ctl->t < ctl->tf) {
                ctl->h = fmin(ctl->dt, ctl->tf - ctl->t);
                ctl->done = 0;
            } else {
                ctl->done = 1;
            }
        }
        grid.sync();
        if (threadIdx.x == 0) s_h = ((volatile Ctl*)ctl)->done ? -1.0 : ((volatile Ctl*)ctl)->h;
        __syncthreads();
        const double h = s_h;
        if (h < 0.0) return;   // uniform over the grid
        TRACE();
        for (int stage = 0; stage < 4; ++stage) {
            for (int it = blockIdx.x; it < na; it += gridDim.x) phase_a<T>(g, it * RA, stage, h, smem);
            TRACE();
            grid.sync();
            TRACE();
            for (int it = blockIdx.x; it < nb; it += gridDim.x) phase_b<T>(g, it * g.CB, g.CB, smem);
            TRACE();
            grid.sync();
            TRACE();
            for (int it = blockIdx.x; it < nc; it += gridDim.x) phase_c<T>(g, it * RC, (T*)g.raw[stage], smem);
            TRACE();
            grid.sync();
            TRACE();
        }
        // phase D: x += h/6 (k1 + 2 k2 + 2 k3 + k4), w = x (+ hi/lo copy)
        __shared__ double s_c[5];
        if (threadIdx.x == 0) {
            s_c[0] = h / 6;
            for (int s = 0; s < 4; ++s) s_c[1 + s] = corner_mean_of((const T*)g.raw[s], nx, ny);
        }
        __syncthreads();
        const T* r1 = (const T*)g.raw[0];
        const T* r2 = (const T*)g.raw[1];
        const T* r3 = (const T*)g.raw[2];
        const T* r4 = (const T*)g.raw[3];
#pragma unroll 4
        for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
            if constexpr (std::is_same<T, float>::value) {
                const float k = ((((float)r1[e] - (float)s_c[1]) + 2.f * ((float)r2[e] - (float)s_c[2])) +
                                 2.f * ((float)r3[e] - (float)s_c[3])) + ((float)r4[e] - (float)s_c[4]);
                const double v = g.x[e] + (double)(k * (float)(s_c[0] * g.spy));
                g.x[e] = v;
                g.w[e] = v;
                const float hi = (float)v;
                g.xhi[e] = hi;
                g.xlo[e] = (float)(v - (double)hi);
            } else {
                const double k1 = ((double)r1[e] - s_c[1]) * g.spy, k2 = ((double)r2[e] - s_c[2]) * g.spy;
                const double k3 = ((double)r3[e] - s_c[3]) * g.spy, k4 = ((double)r4[e] - s_c[4]) * g.spy;
                const double v = g.x[e] + s_c[0] * (((k1 + 2 * k2) + 2 * k3) + k4);
                g.x[e] = v;
                g.w[e] = v;
            }
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->t = ctl->t + h;
            ctl->n_accept++;
        }
        TRACE();
        grid.sync();
        TRACE();
    }
#undef TRACE
}

// hi/lo split of the double state (mixed form), used before the first step
// and after anything outside the engine changed x or w_ref.
__global__ void k_split(const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const double v = x[e];
        const float a = (float)v;
        hi[e] = a;
        lo[e] = (float)(v - (double)a);
    }
}

void split_hilo(const double* x, float* hi, float* lo, size_t n, cudaStream_t s)
{
    int b = (int)((n + 255) / 256);
    if (b > 1216) b = 1216;
    k_split<<<b, 256, 0, s>>>(x, hi, lo, n);
}

static int engine_bps()
{
    const char* e = getenv("FI_ENGINE_BPS");
    return (e && e[0] == '2') ? 2 : 1;
}

template <typename T> int engine_config(const Plan2D& p, int* grid, int* CB, size_t* smem)
{
    typedef typename vec2<T>::type C2;
    if (p.nx % 4 != 0) return 0;   // 16-byte row vectors in the phase-A prefetch
    int cb = (int)(16 / sizeof(C2));
    if (cb < 1) cb = 1;
    *CB = cb;
    *smem = engine_smem_bytes<T>(p, cb);
    int dev = 0, nsm = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (*smem > (size_t)optin) return 0;
    const int bps = engine_bps();
    cudaError_t e1 = bps == 2 ? cudaFuncSetAttribute(k_engine_rk4<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem)
                              : cudaFuncSetAttribute(k_engine_rk4<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
    if (e1 != cudaSuccess) return 0;
    int per_sm = 0;
    cudaError_t e2 = bps == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_engine_rk4<T, 2>, 256, *smem)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_engine_rk4<T, 1>, 256, *smem);
    if (e2 != cudaSuccess || per_sm < 1) return 0;
    if (per_sm > bps) per_sm = bps;
    *grid = per_sm * nsm;
    return 1;
}

template <typename T> cudaError_t engine_launch(const EngineArgs& g, int grid, size_t smem, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (engine_bps() == 2) return cudaLaunchKernelEx(&cfg, k_engine_rk4<T, 2>, g);
    return cudaLaunchKernelEx(&cfg, k_engine_rk4<T, 1>, g);
}

template size_t engine_smem_bytes<float>(const Plan2D&, int);
template size_t engine_smem_bytes<double>(const Plan2D&, int);
template int engine_config<float>(const Plan2D&, int*, int*, size_t*);
template int engine_config<double>(const Plan2D&, int*, int*, size_t*);
template cudaError_t engine_launch<float>(const EngineArgs&, int, size_t, cudaStream_t);
template cudaError_t engine_launch<double>(const EngineArgs&, int, size_t, cudaStream_t);

}  // namespace fi
