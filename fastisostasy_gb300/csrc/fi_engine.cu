// fi_engine.cu — persistent cooperative RK4 step engine.
//
// One cooperative launch integrates all RK4 steps of an isos_update
// (step_rk4 with true stages, src/integrators.f90:42-77, evaluating
// calc_lvelva, src/lv_elva.f90:31-126, at every stage state).  The grid
// walks through phases separated by grid-wide barriers:
//
//   S  flexure stencil on 64 x 16 tiles -> f
//   R  forward row real-FFT, one warp per row -> half spectrum
//   C  column FFT, multiply by 1/(kappa R) in the Hartley basis, inverse (one warp per column)
//   I  inverse row real-FFT, one warp per row -> raw_s (stage output before corner BC / sec_per_year)
//   D  x += h/6 (k1 + 2 k2 + 2 k3 + k4), w = x
//
// Stage states y_s = x + a_s h k_{s-1} are never stored: phase S rebuilds the
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
#include "fi_wfft.cuh"

namespace cg = cooperative_groups;

namespace fi {

template <typename T> __device__ __forceinline__ const typename vec2<T>::type* etw(const FftLen& L);
template <> __device__ __forceinline__ const double2* etw<double>(const FftLen& L) { return L.tw64; }
template <> __device__ __forceinline__ const float2* etw<float>(const FftLen& L) { return L.tw32; }
template <typename T> __device__ __forceinline__ const typename vec2<T>::type* ertw(const Plan2D& p);
template <> __device__ __forceinline__ const double2* ertw<double>(const Plan2D& p) { return p.rtw64; }
template <> __device__ __forceinline__ const float2* ertw<float>(const Plan2D& p) { return p.rtw32; }

__device__ __forceinline__ unsigned long long gtimer0()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// stage coefficients of RK4: y_s = x + a_s h k_{s-1}
__constant__ double c_rk4_a[4] = {0.0, 0.5, 0.5, 1.0};

// ---------------------------------------------------------------------------
// Stencil tiles: SX x SY outputs per item, halo 2; 256 threads as 64 x 4, each
// thread owning one column and four output rows.
// ---------------------------------------------------------------------------
constexpr int SX = 64, SY = 16, SRX = SX + 4, SRY = SY + 4, SREG = SRX * SRY;
constexpr int ENGINE_THREADS = 256, ENGINE_WARPS = ENGINE_THREADS / 32;

constexpr int RB = 4;   // rows per row-phase item (one warp per row; 32-byte transpose segments)

template <typename T> size_t engine_smem_bytes(const Plan2D& p, int)
{
    typedef typename vec2<T>::type C2;
    const size_t nw = (sizeof(T) == 4) ? 4 : 3;   // interior arrays: q0, 1/(2 eta), w_ref (hi, lo)
    const size_t stencil = (size_t)11 * SREG * sizeof(T) + nw * SX * SY * sizeof(T) + SX * SY;
    const size_t rows = (size_t)RB * (p.h + 1) * sizeof(C2) + (size_t)ENGINE_WARPS * p.h * sizeof(C2);
    const size_t cols = (size_t)ENGINE_WARPS * p.ny * sizeof(C2);
    size_t m = stencil > rows ? stencil : rows;
    m = m > cols ? m : cols;
    return m + 64;
}

template <typename T>
__device__ void phase_stencil(const EngineArgs& g, int tile, int stage, double h, unsigned char* smem)
{
    const int nx = g.p.nx, ny = g.p.ny;
    const int ntx = (nx + SX - 1) / SX;
    const int i0 = (tile % ntx) * SX - 2, j0 = (tile / ntx) * SY - 2;   // global index of local (0, 0)
    const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;
    T* A0 = reinterpret_cast<T*>(smem);   // mixed: x hi | plain: x
    T* A1 = A0 + SREG;                    // mixed: x lo | plain: raw_prev
    T* A2 = A1 + SREG;                    // mixed: raw_prev | plain: y
    T* dX = A2 + SREG;
    T* dY = dX + SREG;
    T* Wx = dY + SREG;
    T* Mxx = Wx + SREG;
    T* Myy = Mxx + SREG;
    T* Mxy = Myy + SREG;
    T* Mxyx = Mxy + SREG;
    T* Ds = Mxyx + SREG;                  // rigidity on the halo region
    T* Qs = Ds + SREG;                    // interior SX x SY arrays
    T* Es = Qs + SX * SY;
    T* W0 = Es + SX * SY;                 // mixed: w_ref hi | plain: w_ref
    T* W1 = W0 + SX * SY;                 // mixed: w_ref lo
    uint8_t* Ks = reinterpret_cast<uint8_t*>(W0 + (sizeof(T) == 4 ? 2 : 1) * SX * SY);
    const T* rprev = stage > 0 ? (const T*)g.raw[stage - 1] : nullptr;
    __shared__ double s_sc[2];
    __syncthreads();   // previous item's readers are done with the tile buffers
    if (threadIdx.x == 0) {
        s_sc[0] = stage > 0 ? c_rk4_a[stage] * h * g.spy : 0.0;
        s_sc[1] = stage > 0 ? corner_mean_of(rprev, nx, ny) : 0.0;
    }
    // every global read of the item in one batch
    const T* Dg = g.D_T<T>();
#pragma unroll
    for (int ly = ty; ly < SRY; ly += 4)
#pragma unroll
        for (int lx = tx; lx < SRX; lx += 64) {
            const int gi = i0 + lx, gj = j0 + ly;
            const int l = ly * SRX + lx;
            T a0 = (T)0, a1 = (T)0, a2 = (T)0, d = (T)0;
            if (gi >= 0 && gi < nx && gj >= 0 && gj < ny) {
                const size_t c = (size_t)gj * nx + gi;
                if constexpr (std::is_same<T, float>::value) {
                    a0 = g.xhi[c];
                    a1 = g.xlo[c];
                    if (rprev) a2 = rprev[c];
                } else {
                    a0 = g.x[c];
                    if (rprev) a1 = rprev[c];
                }
                d = __ldg(Dg + c);
            }
            A0[l] = a0;
            A1[l] = a1;
            A2[l] = a2;
            Ds[l] = d;
        }
    {
        const T* q0 = g.q0_T<T>();
        const T* i2e = g.inv2eta_T<T>();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int oy = ty + 4 * q;
            const int gi = i0 + 2 + tx, gj = j0 + 2 + oy;
            const int o = oy * SX + tx;
            T qv = (T)0, ev = (T)0, w0 = (T)0, w1 = (T)0;
            uint8_t mk = 0;
            if (gi < nx && gj < ny) {
                const size_t c = (size_t)gj * nx + gi;
                qv = __ldg(q0 + c);
                ev = __ldg(i2e + c);
                mk = g.mask[c];
                if constexpr (std::is_same<T, float>::value) {
                    w0 = __ldg(g.wrefhi + c);
                    w1 = __ldg(g.wreflo + c);
                } else {
                    w0 = __ldg(g.wref + c);
                }
            }
            Qs[o] = qv;
            Es[o] = ev;
            W0[o] = w0;
            if constexpr (std::is_same<T, float>::value) W1[o] = w1;
            Ks[o] = mk;
        }
    }
    __syncthreads();
    const double sd = s_sc[0], cmd = s_sc[1];
    const float sf = (float)sd;
    if constexpr (!std::is_same<T, float>::value) {
        // plain form: the stage state y = x + s (raw - cm) in double
        for (int e = threadIdx.x; e < SREG; e += ENGINE_THREADS) A2[e] = rprev ? A0[e] + sd * (A1[e] - cmd) : A0[e];
        __syncthreads();
    }
#pragma unroll
    for (int ly = ty; ly < SRY; ly += 4)
#pragma unroll
        for (int lx = tx; lx < SRX; lx += 64) {
            const int l = ly * SRX + lx;
            if (lx < SRX - 1) {
                if constexpr (std::is_same<T, float>::value)
                    dX[l] = (A0[l + 1] - A0[l]) + (A1[l + 1] - A1[l]) + sf * (A2[l + 1] - A2[l]);
                else
                    dX[l] = A2[l + 1] - A2[l];
            }
            if (ly < SRY - 1) {
                if constexpr (std::is_same<T, float>::value)
                    dY[l] = (A0[l + SRX] - A0[l]) + (A1[l + SRX] - A1[l]) + sf * (A2[l + SRX] - A2[l]);
                else
                    dY[l] = A2[l + SRX] - A2[l];
            }
        }
    __syncthreads();
    const T inv_dx = (T)g.fc.inv_dx, inv_2dx = (T)g.fc.inv_2dx, inv_dx2 = (T)g.fc.inv_dx2;
    const T inv_dy = (T)g.fc.inv_dy, inv_2dy = (T)g.fc.inv_2dy, inv_dy2 = (T)g.fc.inv_dy2;
#pragma unroll
    for (int ly = ty; ly < SRY; ly += 4)
#pragma unroll
        for (int lx = tx + 1; lx < SRX - 1; lx += 64) {
            const int gi = i0 + lx;
            const int l = ly * SRX + lx;
            T v;
            if (gi == 0) v = dX[l] * inv_dx;
            else if (gi == nx - 1) v = dX[l - 1] * inv_dx;
            else v = (dX[l] + dX[l - 1]) * inv_2dx;
            Wx[l] = v;
        }
    __syncthreads();
    const T nu = (T)g.fc.nu, omn = (T)g.fc.one_minus_nu;
#pragma unroll
    for (int ly = ty + 1; ly < SRY - 1; ly += 4)
#pragma unroll
        for (int lx = tx + 1; lx < SRX - 1; lx += 64) {
            const int gi = i0 + lx, gj = j0 + ly;
            if (gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
            const int l = ly * SRX + lx;
            T wxy, wxx, wyy;
            if (gj == 0) wxy = (Wx[l + SRX] - Wx[l]) * inv_dy;
            else if (gj == ny - 1) wxy = (Wx[l] - Wx[l - SRX]) * inv_dy;
            else wxy = (Wx[l + SRX] - Wx[l - SRX]) * inv_2dy;
            if (gi == 0) wxx = (dX[l + 1] - dX[l]) * inv_dx2;
            else if (gi == nx - 1) wxx = (dX[l - 1] - dX[l - 2]) * inv_dx2;
            else wxx = (dX[l] - dX[l - 1]) * inv_dx2;
            if (gj == 0) wyy = (dY[l + SRX] - dY[l]) * inv_dy2;
            else if (gj == ny - 1) wyy = (dY[l - SRX] - dY[l - 2 * SRX]) * inv_dy2;
            else wyy = (dY[l] - dY[l - SRX]) * inv_dy2;
            const T Dl = Ds[l];
            Mxx[l] = -Dl * (wxx + nu * wyy);
            Myy[l] = -Dl * (wyy + nu * wxx);
            Mxy[l] = (-Dl * omn) * wxy;
        }
    __syncthreads();
#pragma unroll
    for (int ly = ty + 1; ly < SRY - 1; ly += 4)
#pragma unroll
        for (int lx = tx + 2; lx < SRX - 2; lx += 64) {
            const int gi = i0 + lx, gj = j0 + ly;
            if (gi < 0 || gi >= nx || gj < 0 || gj >= ny) continue;
            const int l = ly * SRX + lx;
            T v;
            if (gi == 0) v = (Mxy[l + 1] - Mxy[l]) * inv_dx;
            else if (gi == nx - 1) v = (Mxy[l] - Mxy[l - 1]) * inv_dx;
            else v = (Mxy[l + 1] - Mxy[l - 1]) * inv_2dx;
            Mxyx[l] = v;
        }
    __syncthreads();
    T* f = (T*)g.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int oy = ty + 4 * q;
        const int lx = tx + 2, ly = oy + 2;
        const int gi = i0 + lx, gj = j0 + ly;
        if (gi >= nx || gj >= ny) continue;
        const int l = ly * SRX + lx, o = oy * SX + tx;
        T mxy_xy, mx_xx, my_yy;
        if (gj == 0) mxy_xy = (Mxyx[l + SRX] - Mxyx[l]) * inv_dy;
        else if (gj == ny - 1) mxy_xy = (Mxyx[l] - Mxyx[l - SRX]) * inv_dy;
        else mxy_xy = (Mxyx[l + SRX] - Mxyx[l - SRX]) * inv_2dy;
        if (gi == 0) mx_xx = ((Mxx[l + 2] - (T)2 * Mxx[l + 1]) + Mxx[l]) * inv_dx2;
        else if (gi == nx - 1) mx_xx = ((Mxx[l] - (T)2 * Mxx[l - 1]) + Mxx[l - 2]) * inv_dx2;
        else mx_xx = ((Mxx[l + 1] - (T)2 * Mxx[l]) + Mxx[l - 1]) * inv_dx2;
        if (gj == 0) my_yy = ((Myy[l + 2 * SRX] - (T)2 * Myy[l + SRX]) + Myy[l]) * inv_dy2;
        else if (gj == ny - 1) my_yy = ((Myy[l] - (T)2 * Myy[l - SRX]) + Myy[l - 2 * SRX]) * inv_dy2;
        else my_yy = ((Myy[l + SRX] - (T)2 * Myy[l]) + Myy[l - SRX]) * inv_dy2;
        T p = (T)0;
        if (Ks[o]) {
            // q0 + (-g rho_m) (y - w_ref) at the stage state
            if constexpr (std::is_same<T, float>::value) {
                float dy = (A0[l] - W0[o]) + (A1[l] - W1[o]);
                if (rprev) dy += sf * (A2[l] - (float)cmd);
                p = Qs[o] + (float)g.fc.coef_mantle * dy;
            } else {
                p = Qs[o] + g.fc.coef_mantle * (A2[l] - W0[o]);
            }
        }
        f[(size_t)gj * nx + gi] = (((p + mx_xx) + (T)2 * mxy_xy) + my_yy) * Es[o];
    }
}

// ---------------------------------------------------------------------------
// Warp-level transforms.  The engine keeps the half spectrum transposed,
// ST[k * ny + l] (k <= h, l < ny), so that every column is contiguous; the
// row phases move 8-row strips through shared memory (64-byte segments).
// ---------------------------------------------------------------------------
template <typename T, int P>
__device__ void rows_fwd_item(const EngineArgs& g, int j0, unsigned char* smem)
{
    typedef typename vec2<T>::type C2;
    constexpr int hh = 32 * P;
    const int ny = g.p.ny;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    C2* X = reinterpret_cast<C2*>(smem);            // RB x (hh+1)
    C2* wb = X + (size_t)RB * (hh + 1) + (size_t)w * hh;
    const int j = j0 + w;
    if (w < RB && j < ny) {
        const C2* f2 = reinterpret_cast<const C2*>((const T*)g.f + (size_t)j * g.p.nx);
        C2 v[P];
#pragma unroll
        for (int p = 0; p < P; ++p) v[p] = f2[lane + 32 * p];
        const C2* rtw = ertw<T>(g.p);
        C2 rt[P + 1];
#pragma unroll
        for (int jj = 0; jj <= P; ++jj) {
            const int k = lane + 32 * jj;
            rt[jj] = k <= hh ? __ldg(rtw + k) : mk2<T>((T)0, (T)0);
        }
        warp_fft<T, P>(v, lane, etw<T>(g.p.row), -1);
        const int base = P * brev5(lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) wb[base + k1] = v[k1];
        __syncwarp();
        C2* Xr = X + (size_t)w * (hh + 1);
#pragma unroll
        for (int jj = 0; jj <= P; ++jj) {
            const int k = lane + 32 * jj;
            if (k <= hh) {
                const C2 Zk = wb[k == hh ? 0 : k];
                const C2 Zc = wb[k == 0 ? 0 : hh - k];
                C2 E, O;
                E.x = (T)0.5 * (Zk.x + Zc.x);
                E.y = (T)0.5 * (Zk.y - Zc.y);
                O.x = (T)0.5 * (Zk.y + Zc.y);
                O.y = (T)-0.5 * (Zk.x - Zc.x);
                Xr[k] = cadd(E, cmul(rt[jj], O));
            }
        }
    }
    __syncthreads();
    C2* ST = (C2*)g.ST;
    for (int e = threadIdx.x; e < RB * (hh + 1); e += ENGINE_THREADS) {
        const int k = e / RB, o = e - k * RB;
        if (j0 + o < ny) ST[(size_t)k * ny + j0 + o] = X[(size_t)o * (hh + 1) + k];
    }
    __syncthreads();
}

template <typename T, int Q>
__device__ void col_w(const EngineArgs& g, int k, typename vec2<T>::type* wb)
{
    typedef typename vec2<T>::type C2;
    constexpr int ny = 32 * Q;
    const int lane = threadIdx.x & 31;
    const bool tr = g.trace && k == 0 && lane == 0 && g.trace[63] == 0;
    unsigned long long tt[8];
    int nt_ = 0;
    if (tr) tt[nt_++] = gtimer0();
    C2* col = (C2*)g.ST + (size_t)k * ny;
    const T* mA = g.mA_T<T>() + (size_t)k * ny;
    const T* mB = g.mB_T<T>() + (size_t)k * ny;
    C2 v[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = col[lane + 32 * q];
    // multipliers of this lane's Hartley pairs (l, ny - l), l = lane + 32 jj <= ny/2
    T ma[Q / 2 + 1], mb[Q / 2 + 1], mc[Q / 2 + 1], md[Q / 2 + 1];
#pragma unroll
    for (int jj = 0; jj <= Q / 2; ++jj) {
        const int l = lane + 32 * jj;
        const int lm = (ny - l) & (ny - 1);
        const bool ok = l <= ny / 2;
        ma[jj] = ok ? __ldg(mA + l) : (T)0;
        mb[jj] = ok ? __ldg(mA + lm) : (T)0;
        mc[jj] = (ok && !g.even) ? __ldg(mB + l) : (T)0;
        md[jj] = (ok && !g.even) ? __ldg(mB + lm) : (T)0;
    }
    if (tr) { volatile float sink = v[0].x + ma[0]; (void)sink; tt[nt_++] = gtimer0(); }
    warp_fft<T, Q>(v, lane, etw<T>(g.p.col), -1);
    if (tr) { volatile float sink = v[0].x; (void)sink; tt[nt_++] = gtimer0(); }
    const int base = Q * brev5(lane);
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) wb[base + k1] = v[k1];
    __syncwarp();
#pragma unroll
    for (int jj = 0; jj <= Q / 2; ++jj) {
        const int l = lane + 32 * jj;
        if (l > ny / 2) continue;
        const int lm = (ny - l) & (ny - 1);
        const C2 Fa = wb[l], Fb = wb[lm];
        C2 a, b;
        if (g.even) {
            a.x = Fa.x * ma[jj]; a.y = Fa.y * ma[jj];
            b.x = Fb.x * mb[jj]; b.y = Fb.y * mb[jj];
        } else {
            // Hartley values at (k,l), (-k,-l), (-k,l), (k,-l), multiplied, back to the DFT
            const T H_kl = Fb.x - Fa.y, H_mkml = Fb.x + Fa.y;
            const T H_mkl = Fa.x + Fb.y, H_kml = Fa.x - Fb.y;
            const T G_kl = ma[jj] * H_kl, G_kml = mb[jj] * H_kml;
            const T G_mkl = mc[jj] * H_mkl, G_mkml = md[jj] * H_mkml;
            a.x = (T)0.5 * (G_kml + G_mkl);
            a.y = (T)0.5 * (G_mkml - G_kl);
            b.x = (T)0.5 * (G_kl + G_mkml);
            b.y = (T)0.5 * (G_mkl - G_kml);
        }
        wb[l] = a;
        if (lm != l) wb[lm] = b;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = wb[lane + 32 * q];
    if (tr) { volatile float sink = v[0].x; (void)sink; tt[nt_++] = gtimer0(); }
    warp_fft<T, Q>(v, lane, etw<T>(g.p.col), +1);
    if (tr) { volatile float sink = v[0].x; (void)sink; tt[nt_++] = gtimer0(); }
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) col[base + k1] = v[k1];
    __syncwarp();
    if (tr) {
        tt[nt_++] = gtimer0();
        for (int i = 0; i < nt_; ++i) g.trace[48 + i] = tt[i];
        g.trace[63] = 1;
    }
}

template <typename T, int P>
__device__ void rows_inv_item(const EngineArgs& g, int j0, T* out, unsigned char* smem)
{
    typedef typename vec2<T>::type C2;
    constexpr int hh = 32 * P;
    const int ny = g.p.ny;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    C2* X = reinterpret_cast<C2*>(smem);            // RB x (hh+1)
    const C2* ST = (const C2*)g.ST;
    {
        constexpr int U = 4;
        const int tot = RB * (hh + 1);
        for (int e0 = threadIdx.x; e0 < tot; e0 += U * ENGINE_THREADS) {
            C2 t[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = e0 + u * ENGINE_THREADS;
                const int k = e / RB, o = e - k * RB;
                t[u] = (e < tot && j0 + o < ny) ? ST[(size_t)k * ny + j0 + o] : mk2<T>((T)0, (T)0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = e0 + u * ENGINE_THREADS;
                const int k = e / RB, o = e - k * RB;
                if (e < tot) X[(size_t)o * (hh + 1) + k] = t[u];
            }
        }
    }
    __syncthreads();
    const int j = j0 + w;
    if (w < RB && j < ny) {
        const C2* Xr = X + (size_t)w * (hh + 1);
        const C2* rtw = ertw<T>(g.p);
        C2 v[P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const int k = lane + 32 * p;
            const C2 A = Xr[k];
            C2 B = Xr[hh - k];
            B.y = -B.y;
            const C2 sum = cadd(A, B), dif = csub(A, B);
            const C2 t = cmulc(dif, __ldg(rtw + k));
            v[p].x = sum.x - t.y;
            v[p].y = sum.y + t.x;
        }
        warp_fft<T, P>(v, lane, etw<T>(g.p.row), +1);
        const T scale = (T)g.norm_scale;
        C2* o = reinterpret_cast<C2*>(out + (size_t)j * g.p.nx) + P * brev5(lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            C2 q = v[k1];
            q.x *= scale;
            q.y *= scale;
            o[k1] = q;
        }
    }
    __syncthreads();
}

// Row/column transform lengths are template parameters (h = 32 P, ny = 32 Q):
// one engine instantiation carries only the code of its own lengths, which
// keeps the kernel small enough for the instruction cache.
template <typename T, int P>
__device__ void phase_rows_fwd(const EngineArgs& g, unsigned char* smem)
{
    const int items = (g.p.ny + RB - 1) / RB;
    for (int it = blockIdx.x; it < items; it += gridDim.x) rows_fwd_item<T, P>(g, it * RB, smem);
}

template <typename T, int Q>
__device__ void phase_cols(const EngineArgs& g, unsigned char* smem)
{
    typedef typename vec2<T>::type C2;
    const int warp = threadIdx.x >> 5;
    C2* wb = reinterpret_cast<C2*>(smem) + (size_t)warp * g.p.ny;
    // one column per block first, so that every SM gets work
    for (int k = blockIdx.x + gridDim.x * warp; k <= g.p.h; k += gridDim.x * ENGINE_WARPS) col_w<T, Q>(g, k, wb);
}

template <typename T, int P>
__device__ void phase_rows_inv(const EngineArgs& g, T* out, unsigned char* smem)
{
    const int items = (g.p.ny + RB - 1) / RB;
    for (int it = blockIdx.x; it < items; it += gridDim.x) rows_inv_item<T, P>(g, it * RB, out, smem);
}

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// MINB blocks per SM: 2 caps the registers at 128 per thread
template <typename T, int P, int Q>
__global__ void __launch_bounds__(256, 2) k_engine_rk4(EngineArgs g)
{
    extern __shared__ __align__(16) unsigned char smem[];
    cg::grid_group grid = cg::this_grid();
    const int nx = g.p.nx, ny = g.p.ny;
    const size_t n = (size_t)nx * ny;
    const int ntiles = ((nx + SX - 1) / SX) * ((ny + SY - 1) / SY);
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
            for (int it = blockIdx.x; it < ntiles; it += gridDim.x) phase_stencil<T>(g, it, stage, h, smem);
            TRACE();
            grid.sync();
            TRACE();
            phase_rows_fwd<T, P>(g, smem);
            TRACE();
            grid.sync();
            TRACE();
            phase_cols<T, Q>(g, smem);
            TRACE();
            grid.sync();
            TRACE();
            phase_rows_inv<T, P>(g, (T*)g.raw[stage], smem);
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

typedef void (*EngineKernel)(EngineArgs);

// h/32 and ny/32 in {4, 8, 16}
template <typename T> EngineKernel engine_kernel(int P, int Q)
{
#define EK(p, q) if (P == p && Q == q) return k_engine_rk4<T, p, q>;
    EK(4, 4) EK(4, 8) EK(4, 16) EK(8, 4) EK(8, 8) EK(8, 16) EK(16, 4) EK(16, 8) EK(16, 16)
#undef EK
    return nullptr;
}

template <typename T> int engine_config(const Plan2D& p, int* grid, int* CB, size_t* smem)
{
    // The plain FP64 form is FP64-throughput bound; it runs faster as the
    // multi-kernel graph (full occupancy) than in the one-grid engine.
    if (sizeof(T) == 8) return 0;
    if (p.h % 32 || p.ny % 32) return 0;
    EngineKernel k = engine_kernel<T>(p.h / 32, p.ny / 32);
    if (!k) return 0;
    *CB = 1;
    *smem = engine_smem_bytes<T>(p, 1);
    int dev = 0, nsm = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (*smem > (size_t)optin) return 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, *smem) != cudaSuccess || per_sm < 1) return 0;
    if (per_sm > 2) per_sm = 2;
    *grid = per_sm * nsm;
    return 1;
}

template <typename T> cudaError_t engine_launch(const EngineArgs& g, int grid, size_t smem, cudaStream_t s)
{
    EngineKernel k = engine_kernel<T>(g.p.h / 32, g.p.ny / 32);
    if (!k) return cudaErrorInvalidValue;
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
    return cudaLaunchKernelEx(&cfg, k, g);
}

template size_t engine_smem_bytes<float>(const Plan2D&, int);
template size_t engine_smem_bytes<double>(const Plan2D&, int);
template int engine_config<float>(const Plan2D&, int*, int*, size_t*);
template <> EngineKernel engine_kernel<double>(int, int) { return nullptr; }
template int engine_config<double>(const Plan2D&, int*, int*, size_t*);
template cudaError_t engine_launch<float>(const EngineArgs&, int, size_t, cudaStream_t);
template cudaError_t engine_launch<double>(const EngineArgs&, int, size_t, cudaStream_t);

}  // namespace fi
