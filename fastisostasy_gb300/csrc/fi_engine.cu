// fi_engine.cu — persistent cooperative RK4 step engine.
//
// One cooperative launch integrates all RK4 steps of an isos_update
// (step_rk4 with true stages, src/integrators.f90:42-77, evaluating
// calc_lvelva, src/lv_elva.f90:31-126, at every stage state).  The grid
// walks through phases separated by grid-wide barriers:
//
//   A  stencil + row real-FFT   (work item = 4 grid rows, full width)
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
#include <mutex>
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

// Rows per phase-A and phase-C item, a template parameter of the kernel
// (even: see the y-boundary stencils).  RA = 4 on one 1024-thread block per
// SM reads 8 state rows for 4 output rows; RA = 2 on two 512-thread blocks
// per SM reads 12, but has twice the items.  The 4-row shape is taken when
// its items occupy most SMs (512^2: 1.198 against 1.251 ms per update), the
// 2-row shape below that (256^2: 128 two-row items against 64 four-row ones).
template <int RA> struct EngShape {
    static constexpr int threads = RA == 4 ? 1024 : 512;
    static constexpr int per_sm = RA == 4 ? 1 : 2;   // resident blocks per SM
    static constexpr int cb = RA == 4 ? 2 : 1;       // spectrum columns per phase-B item
};

// stage coefficients of RK4: y_s = x + a_s h k_{s-1}
__constant__ double c_rk4_a[4] = {0.0, 0.5, 0.5, 1.0};

template <typename T, int RA> struct PhaseAMem {
    // level-0 differences on RA+4 rows, moments on RA+2 rows, all full width
    __host__ __device__ static size_t bytes(int nx, int h)
    {
        typedef typename vec2<T>::type C2;
        const size_t rows = (RA + 4) + (RA + 3) + (RA + 4) + 4 * (RA + 2);
        return rows * (size_t)nx * sizeof(T) + 2 * (size_t)RA * h * sizeof(C2);
    }
};

// Dynamic shared memory: the phase scratch (the largest of A, B, C), then
// the twiddle tables of the row and column transforms and of the real-FFT
// split, copied once per launch and resident for all its phases.
template <typename T, int RA> __host__ __device__ inline size_t engine_tab_off(int nx, int h, int ny, int CB)
{
    typedef typename vec2<T>::type C2;
    constexpr int RC = RA;
    const size_t a = PhaseAMem<T, RA>::bytes(nx, h);
    const size_t b = 2 * (size_t)CB * ny * sizeof(C2);
    const size_t c = 2 * (size_t)RC * h * sizeof(C2);
    size_t m = a > b ? a : b;
    m = m > c ? m : c;
    return (m + 15) & ~(size_t)15;
}
template <typename T> __host__ __device__ inline size_t engine_tab_count(int h, int ny)
{
    return (size_t)h + (size_t)ny + (size_t)h + 1;   // row, column, real split
}

template <typename T, int RA> size_t engine_smem_bytes(const Plan2D& p, int CB)
{
    typedef typename vec2<T>::type C2;
    return engine_tab_off<T, RA>(p.nx, p.h, p.ny, CB) + engine_tab_count<T>(p.h, p.ny) * sizeof(C2) + 64;
}

// (row, column) walk of a block's threads over a row-major strip of width w
// in steps of the block size: the element index e = r*w + i advances by nt
// without a per-element integer division (a runtime division is a long
// instruction sequence and the strip loops of phase A are issue-bound).
struct Walk {
    int r0, i0, dr, di, w;
    __device__ __forceinline__ void init(int width, int tid, int nt)
    {
        w = width;
        r0 = tid / width;
        i0 = tid - r0 * width;
        dr = nt / width;
        di = nt - dr * width;
    }
    __device__ __forceinline__ void next(int& r, int& i) const
    {
        i += di;
        r += dr;
        if (i >= w) {
            i -= w;
            ++r;
        }
    }
};

// per-launch constants of a block: resident twiddle tables and strip walks
template <typename T> struct EngTw {
    const typename vec2<T>::type* row;
    const typename vec2<T>::type* col;
    const typename vec2<T>::type* rtw;
    Walk wx;    // width nx (phase A strips)
    Walk wh;    // width h (phase C rows)
    Walk wh1;   // width h+1 (half-spectrum rows)
};

template <typename T> __device__ __forceinline__ double corner_mean_dev(const T* a, int nx, int ny)
{
    return corner_mean_of(a, nx, ny);
}

// Phase tracing (fi_engine_trace): block 0 stamps %globaltimer at phase and
// sub-phase boundaries of the first RK4 step; s_trk < 0 when not tracing.
__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__shared__ int s_trk;
constexpr int kTraceLen = 256;
__device__ __forceinline__ void tmark(unsigned long long* tr)
{
    if (threadIdx.x == 0 && s_trk >= 0 && s_trk < kTraceLen) tr[s_trk++] = gtimer();
}

// ---------------------------------------------------------------------------
// Phase A: one item = output rows j0 .. j0+RA-1 (full width).
// ---------------------------------------------------------------------------
template <typename T, int RA, int FM>
__device__ void phase_a(const EngineArgs& g, int j0, int stage, float sdf_in, unsigned char* smem,
                        const EngTw<T>& tw)
{
    static_assert(std::is_same<T, float>::value, "the step engine runs the mixed form only");
    typedef typename vec2<T>::type C2;
    const int nx = g.p.nx, ny = g.p.ny, hh = g.p.h;
    const int tid = threadIdx.x;
    T* dX = reinterpret_cast<T*>(smem);
    T* dY = dX + (size_t)(RA + 4) * nx;
    T* Wx = dY + (size_t)(RA + 3) * nx;
    T* Mxx = Wx + (size_t)(RA + 4) * nx;
    T* Myy = Mxx + (size_t)(RA + 2) * nx;
    T* Mxy = Myy + (size_t)(RA + 2) * nx;
    T* Mxyx = Mxy + (size_t)(RA + 2) * nx;
    C2* b0 = reinterpret_cast<C2*>(Mxyx + (size_t)(RA + 2) * nx);
    C2* b1 = b0 + (size_t)RA * hh;

    const float* rprev = stage > 0 ? (const float*)g.raw[stage - 1] : nullptr;
    __shared__ float s_cmf;
    // y = x + a h spy (raw - cm): the float scale sdf_in = a h spy and the
    // corner mean cm of raw_{s-1}.  GB300 runs FP64 instructions
    // (conversions included) at 1/64 of the FP32 rate, so no thread but
    // thread 0 executes any here: the scale and the coefficients come in as
    // floats (sdf_in, g.fcf).  cm cancels in the level-0 differences and
    // enters only the mantle term: thread 0 issues the four corner loads now
    // and forms the mean after the level-0 loop, so their L2 latency hides
    // behind it.
    float cf[4] = {0.f, 0.f, 0.f, 0.f};
    if (tid == 0 && rprev) {
        const size_t last = (size_t)(ny - 1) * nx;
        const float* q[4] = {rprev, rprev + last + nx - 1, rprev + last, rprev + nx - 1};
#pragma unroll
        for (int c = 0; c < 4; ++c) asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(cf[c]) : "l"(q[c]));
    }
    const float sdf = sdf_in, cmant = g.fcf.coef_mantle;

    // level 0: forward differences along x (dX) and y (dY)
    for (int r = tw.wx.r0, i = tw.wx.i0; r < RA + 4; tw.wx.next(r, i)) {
        const int gj = j0 - 2 + r;
        if (gj < 0 || gj >= ny) continue;
        const size_t c0 = (size_t)gj * nx + i;
        if (i < nx - 1) {
            float v = (g.xhi[c0 + 1] - g.xhi[c0]) + (g.xlo[c0 + 1] - g.xlo[c0]);
            if (rprev) v += sdf * (rprev[c0 + 1] - rprev[c0]);
            dX[(size_t)r * nx + i] = v;
        }
        if (r < RA + 3 && gj + 1 < ny) {
            const size_t c1 = c0 + nx;
            float v = (g.xhi[c1] - g.xhi[c0]) + (g.xlo[c1] - g.xlo[c0]);
            if (rprev) v += sdf * (rprev[c1] - rprev[c0]);
            dY[(size_t)r * nx + i] = v;
        }
    }
    if (tid == 0) s_cmf = rprev ? (float)corner_mean((double)cf[0], (double)cf[1], (double)cf[2], (double)cf[3]) : 0.f;
    __syncthreads();
    tmark(g.trace);
    const float inv_dx = g.fcf.inv_dx, inv_2dx = g.fcf.inv_2dx, inv_dx2 = g.fcf.inv_dx2;
    const float inv_dy = g.fcf.inv_dy, inv_2dy = g.fcf.inv_2dy, inv_dy2 = g.fcf.inv_dy2;
    const float cmdf = s_cmf;
    for (int r = tw.wx.r0, i = tw.wx.i0; r < RA + 4; tw.wx.next(r, i)) {
        const int gj = j0 - 2 + r;
        if (gj < 0 || gj >= ny) continue;
        const float* d = dX + (size_t)r * nx;
        float v;
        if (i == 0) v = d[0] * inv_dx;
        else if (i == nx - 1) v = d[nx - 2] * inv_dx;
        else v = (d[i] + d[i - 1]) * inv_2dx;
        Wx[(size_t)r * nx + i] = v;
    }
    __syncthreads();
    tmark(g.trace);
    const float nu = g.fcf.nu, omn = g.fcf.one_minus_nu;
    for (int m = tw.wx.r0, i = tw.wx.i0; m < RA + 2; tw.wx.next(m, i)) {
        const int r = m + 1;
        const int gj = j0 - 2 + r;
        if (gj < 0 || gj >= ny) continue;
        const size_t ri = (size_t)r * nx + i;
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
        const size_t mi = (size_t)m * nx + i;
        const float Dl = ((const float*)g.D)[(size_t)gj * nx + i];
        Mxx[mi] = -Dl * (wxx + nu * wyy);
        Myy[mi] = -Dl * (wyy + nu * wxx);
        Mxy[mi] = (-Dl * omn) * wxy;
    }
    __syncthreads();
    tmark(g.trace);
    for (int m = tw.wx.r0, i = tw.wx.i0; m < RA + 2; tw.wx.next(m, i)) {
        const int gj = j0 - 1 + m;
        if (gj < 0 || gj >= ny) continue;
        const T* M = Mxy + (size_t)m * nx;
        T v;
        if (i == 0) v = (M[1] - M[0]) * inv_dx;
        else if (i == nx - 1) v = (M[nx - 1] - M[nx - 2]) * inv_dx;
        else v = (M[i + 1] - M[i - 1]) * inv_2dx;
        Mxyx[(size_t)m * nx + i] = v;
    }
    __syncthreads();
    tmark(g.trace);
    for (int o = tw.wx.r0, i = tw.wx.i0; o < RA; tw.wx.next(o, i)) {
        const int gj = j0 + o;
        T fv = (T)0;
        if (gj < ny) {
            const int m = o + 1;
            const size_t mi = (size_t)m * nx + i;
            T mxy_xy, mx_xx, my_yy;
            if (gj == 0) mxy_xy = (Mxyx[mi + nx] - Mxyx[mi]) * inv_dy;
            else if (gj == ny - 1) mxy_xy = (Mxyx[mi] - Mxyx[mi - nx]) * inv_dy;
            else mxy_xy = (Mxyx[mi + nx] - Mxyx[mi - nx]) * inv_2dy;
            const T* M = Mxx + (size_t)m * nx;
            if (i == 0) mx_xx = ((M[2] - (T)2 * M[1]) + M[0]) * inv_dx2;
            else if (i == nx - 1) mx_xx = ((M[nx - 1] - (T)2 * M[nx - 2]) + M[nx - 3]) * inv_dx2;
            else mx_xx = ((M[i + 1] - (T)2 * M[i]) + M[i - 1]) * inv_dx2;
            if (gj == 0) my_yy = ((Myy[mi + 2 * nx] - (T)2 * Myy[mi + nx]) + Myy[mi]) * inv_dy2;
            else if (gj == ny - 1) my_yy = ((Myy[mi] - (T)2 * Myy[mi - nx]) + Myy[mi - 2 * nx]) * inv_dy2;
            else my_yy = ((Myy[mi + nx] - (T)2 * Myy[mi]) + Myy[mi - nx]) * inv_dy2;
            const size_t c = (size_t)gj * nx + i;
            float p = 0.f;
            if (g.mask[c]) {
                // q0 + (-g rho_m) (y - w_ref) with y the stage state
                float dy = (g.xhi[c] - g.wrefhi[c]) + (g.xlo[c] - g.wreflo[c]);
                if (rprev) dy += sdf * (rprev[c] - cmdf);
                p = ((const float*)g.q0)[c] + cmant * dy;
            }
            fv = (((p + mx_xx) + 2.f * mxy_xy) + my_yy) * ((const float*)g.inv2eta)[c];
        }
        // pack the real row as complex pairs for the half-length FFT
        T* bz = reinterpret_cast<T*>(b0 + (size_t)o * hh);
        bz[i] = fv;
    }
    __syncthreads();
    tmark(g.trace);
    C2* r = block_fft<T, true, FM>(b0, b1, g.p.row.d, RA, hh, tw.row, -1);
    const C2* rtw = tw.rtw;
    // column-major: the strided stores do not hold the block up, and phase B
    // then reads each spectrum column contiguously
    C2* ST = (C2*)g.ST;
    for (int o = tw.wh1.r0, k = tw.wh1.i0; o < RA; tw.wh1.next(o, k)) {
        const int gj = j0 + o;
        if (gj >= ny) continue;
        const C2 Zk = r[o * hh + (k == hh ? 0 : k)];
        const C2 Zc = r[o * hh + (k == 0 ? 0 : hh - k)];
        C2 E, O;
        E.x = (T)0.5 * (Zk.x + Zc.x);
        E.y = (T)0.5 * (Zk.y - Zc.y);
        O.x = (T)0.5 * (Zk.y + Zc.y);
        O.y = (T)-0.5 * (Zk.x - Zc.x);
        ST[(size_t)k * ny + gj] = cadd(E, cmul(rtw[k], O));
    }
    __syncthreads();
    tmark(g.trace);
}

// ---------------------------------------------------------------------------
// Phase B: CB spectrum columns: forward column FFT, Hartley-basis multiply,
// inverse column FFT.  Columns come contiguous from the column-major copy
// phase A wrote; the result goes back row-major for the row passes of C.
// ---------------------------------------------------------------------------
template <typename T, int FM>
__device__ void phase_b(const EngineArgs& g, int k0, int CB, unsigned char* smem, const EngTw<T>& tw)
{
    typedef typename vec2<T>::type C2;
    const int ny = g.p.ny;
    C2* b0 = reinterpret_cast<C2*>(smem);
    C2* b1 = b0 + (size_t)CB * ny;
    C2* S = (C2*)g.S;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < CB * ny; e += nt) {
        const int c = CB == 1 ? 0 : e % CB, l = CB == 1 ? e : e / CB;
        const int k = k0 + c;
        b0[c * ny + l] = (k <= g.p.h) ? ((const C2*)g.ST)[(size_t)k * ny + l] : mk2<T>((T)0, (T)0);
    }
    __syncthreads();
    tmark(g.trace);
    C2* r = block_fft<T, true, FM>(b0, b1, g.p.col.d, CB, ny, tw.col, -1);
    const T* mA = g.mA_T<T>();
    const T* mB = g.mB_T<T>();
    const int half = ny / 2 + 1;
    for (int e = tid; e < CB * half; e += nt) {
        const int c = CB == 1 ? 0 : e % CB, l = CB == 1 ? e : e / CB;
        const int k = k0 + c;
        if (k > g.p.h) continue;
        const int lm = (ny - l) % ny;
        C2* col = r + (size_t)c * ny;
        const size_t ia = (size_t)k * ny + l, ib = (size_t)k * ny + lm;   // column-major factors
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
    tmark(g.trace);
    C2* other = (r == b0) ? b1 : b0;
    C2* q = block_fft<T, true, FM>(r, other, g.p.col.d, CB, ny, tw.col, +1);
    for (int e = tid; e < CB * ny; e += nt) {
        const int c = CB == 1 ? 0 : e % CB, l = CB == 1 ? e : e / CB;
        const int k = k0 + c;
        if (k <= g.p.h) S[(size_t)l * g.p.sp + k] = q[c * ny + l];
    }
    __syncthreads();
    tmark(g.trace);
}

// ---------------------------------------------------------------------------
// Phase C: inverse row real-FFT of rows j0 .. j0+RC-1 -> raw (scaled 1/(nx ny)).
// ---------------------------------------------------------------------------
template <typename T, int RC, int FM>
__device__ void phase_c(const EngineArgs& g, int j0, T* out, unsigned char* smem, const EngTw<T>& tw)
{
    typedef typename vec2<T>::type C2;
    const int hh = g.p.h, ny = g.p.ny, nx = g.p.nx;
    C2* b0 = reinterpret_cast<C2*>(smem);
    C2* b1 = b0 + (size_t)RC * hh;
    const C2* S = (const C2*)g.S;
    const C2* rtw = tw.rtw;
    for (int o = tw.wh.r0, k = tw.wh.i0; o < RC; tw.wh.next(o, k)) {
        const int e = o * hh + k;
        const int j = j0 + o;
        C2 z = mk2<T>((T)0, (T)0);
        if (j < ny) {
            const C2 A = S[(size_t)j * g.p.sp + k];
            C2 B = S[(size_t)j * g.p.sp + (hh - k)];
            B.y = -B.y;
            const C2 sum = cadd(A, B), dif = csub(A, B);
            const C2 t = cmulc(dif, rtw[k]);
            z.x = sum.x - t.y;
            z.y = sum.y + t.x;
        }
        b0[e] = z;
    }
    __syncthreads();
    tmark(g.trace);
    C2* r = block_fft<T, true, FM>(b0, b1, g.p.row.d, RC, hh, tw.row, +1);
    T scale;
    if constexpr (std::is_same<T, float>::value) scale = g.norm_scale_f;
    else scale = g.norm_scale;
    for (int o = tw.wh.r0, m = tw.wh.i0; o < RC; tw.wh.next(o, m)) {
        const int j = j0 + o;
        if (j >= ny) continue;
        C2 v = r[o * hh + m];
        v.x *= scale;
        v.y *= scale;
        *reinterpret_cast<C2*>(out + (size_t)j * nx + 2 * m) = v;
    }
    __syncthreads();
    tmark(g.trace);
}

// ---------------------------------------------------------------------------

// Grid barrier of the cooperative launch (every block is resident): after
// the block's barrier, thread 0 arrives with a release add on the launch's
// counter and polls it with acquire loads until all blocks of this barrier
// have arrived (the target grows by gridDim.x per barrier; the counter is
// zeroed before the launch), then releases its block.  The release makes
// the block's writes before the barrier visible at GPU scope to every
// block whose acquire sees the count.  The wait is bounded: past kBarPolls
// polls the block records ST_TIMEOUT and the kernel returns; the blocks
// still waiting then run out of polls as well (bar_phantom > 0 makes every
// wait expire so, for the test of this bound).
constexpr long long kBarPolls = 1ll << 22;
__device__ __forceinline__ bool grid_barrier(const EngineArgs& g, unsigned& target)
{
    __shared__ int s_bar_ok;
    __syncthreads();
    target += gridDim.x + (unsigned)g.bar_phantom;
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(g.bar), "r"(1u) : "memory");
        int ok = 1;
        for (long long polls = 0;; ++polls) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(g.bar) : "memory");
            if (v >= target) break;
            if (polls > kBarPolls) {
                ok = 0;
                g.ctl->status = ST_TIMEOUT;
                break;
            }
        }
        s_bar_ok = ok;
    }
    __syncthreads();
    return s_bar_ok != 0;
}

// FM: the block-FFT index mode, FFT_POW2 when both transform lengths are
// powers of two, else FFT_ANY
template <typename T, int RA, int FM>
__global__ void __launch_bounds__(EngShape<RA>::threads, EngShape<RA>::per_sm) k_engine_rk4(EngineArgs g)
{
    constexpr int RC = RA;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned bar_target = 0;   // arrivals expected at the next grid barrier
    const int nx = g.p.nx, ny = g.p.ny;
    const size_t n = (size_t)nx * ny;
    const int na = (ny + RA - 1) / RA, nb = (g.p.h + 1 + g.CB - 1) / g.CB, nc = (ny + RC - 1) / RC;
    Ctl* ctl = g.ctl;
    // The step control is replicated in every block (the same arithmetic on
    // the same inputs, so every block decides alike) instead of broadcast
    // through a grid barrier; block 0 keeps the control block up to date.
    __shared__ double s_t, s_tf, s_dt;
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        s_t = ctl->t;
        s_tf = ctl->tf;
        s_dt = ctl->dt;
        s_ok = ctl->status == ST_OK;
    }
    // resident twiddle tables (see engine_tab_off)
    typedef typename vec2<T>::type C2;
    EngTw<T> tw;
    {
        C2* tab = reinterpret_cast<C2*>(smem + engine_tab_off<T, RA>(nx, g.p.h, ny, g.CB));
        const C2* srow = etw<T>(g.p.row);
        const C2* scol = etw<T>(g.p.col);
        const C2* srtw = ertw<T>(g.p);
        const int h = g.p.h;
        for (int e = threadIdx.x; e < h; e += blockDim.x) tab[e] = srow[e];
        for (int e = threadIdx.x; e < ny; e += blockDim.x) tab[h + e] = scol[e];
        for (int e = threadIdx.x; e <= h; e += blockDim.x) tab[h + ny + e] = srtw[e];
        tw.row = tab;
        tw.col = tab + h;
        tw.rtw = tab + h + ny;
        tw.wx.init(nx, threadIdx.x, blockDim.x);
        tw.wh.init(h, threadIdx.x, blockDim.x);
        tw.wh1.init(h + 1, threadIdx.x, blockDim.x);
    }
    __syncthreads();
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (threadIdx.x == 0) s_trk = (g.trace && blockIdx.x == 0) ? 0 : -1;
    __syncthreads();
#define TRACE() tmark(g.trace)
    // per-step scalars, computed by thread 0 (the only thread of the mixed
    // form that executes FP64 instructions outside the state update)
    __shared__ int s_go, s_last;
    __shared__ double s_h;
    __shared__ float s_sdf[4];   // float stage scales a_s h spy
    __shared__ float s_cf[5];    // phase D: corner means of raw_1..4 and h/6 spy
    for (int step = 0; step < g.nsteps; ++step) {
        TRACE();
        if (threadIdx.x == 0) {
            const double t = s_t;
            s_go = s_ok && t < s_tf;
            // step_rk4: h = min(dt, tf - t) (src/integrators.f90:62-63)
            const double hh = fmin(s_dt, s_tf - t);
            s_h = hh;
            // now%w is read by nothing inside the engine: written in the last step only
            s_last = step + 1 == g.nsteps || !(t + hh < s_tf);
            for (int st = 0; st < 4; ++st) s_sdf[st] = st > 0 ? (float)(c_rk4_a[st] * hh * g.spy) : 0.f;
        }
        __syncthreads();
        if (!s_go) {   // uniform over the grid
            if (lead) ctl->done = 1;
            return;
        }
        const double h = s_h;
        if (lead) {
            ctl->h = h;
            ctl->done = 0;
        }
        const bool last = s_last != 0;
        TRACE();
        for (int stage = 0; stage < 4; ++stage) {
            for (int it = blockIdx.x; it < na; it += gridDim.x)
                phase_a<T, RA, FM>(g, it * RA, stage, s_sdf[stage], smem, tw);
            TRACE();
            if (!grid_barrier(g, bar_target)) return;
            TRACE();
            for (int it = blockIdx.x; it < nb; it += gridDim.x) phase_b<T, FM>(g, it * g.CB, g.CB, smem, tw);
            TRACE();
            if (!grid_barrier(g, bar_target)) return;
            TRACE();
            for (int it = blockIdx.x; it < nc; it += gridDim.x) phase_c<T, RC, FM>(g, it * RC, (T*)g.raw[stage], smem, tw);
            TRACE();
            if (!grid_barrier(g, bar_target)) return;
            TRACE();
        }
        // phase D: x += h/6 (k1 + 2 k2 + 2 k3 + k4), w = x (+ hi/lo copy)
        __shared__ double s_c[5];
        if (threadIdx.x == 0) {
            s_c[0] = h / 6;
            for (int s = 0; s < 4; ++s) s_c[1 + s] = corner_mean_of((const T*)g.raw[s], nx, ny);
            for (int s = 0; s < 4; ++s) s_cf[s] = (float)s_c[1 + s];
            s_cf[4] = (float)(s_c[0] * g.spy);
        }
        __syncthreads();
        const float c1f = s_cf[0], c2f = s_cf[1], c3f = s_cf[2], c4f = s_cf[3];
        const float scf = s_cf[4];
        const T* r1 = (const T*)g.raw[0];
        const T* r2 = (const T*)g.raw[1];
        const T* r3 = (const T*)g.raw[2];
        const T* r4 = (const T*)g.raw[3];
        for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
            if constexpr (std::is_same<T, float>::value) {
                const float k = ((((float)r1[e] - c1f) + 2.f * ((float)r2[e] - c2f)) + 2.f * ((float)r3[e] - c3f)) +
                                ((float)r4[e] - c4f);
                const float inc = k * scf;
                const double v = g.x[e] + (double)inc;   // the FP64 state update
                g.x[e] = v;
                if (last) g.w[e] = v;
                // the float pair of x takes the same increment by an FP32 two-sum
                const float hi = g.xhi[e], lo = g.xlo[e];
                const float sm = hi + inc, bb = sm - hi;
                const float er = (hi - (sm - bb)) + (inc - bb);
                const float l2 = lo + er;
                const float h2 = sm + l2;
                g.xhi[e] = h2;
                g.xlo[e] = l2 - (h2 - sm);
            } else {
                const double k1 = ((double)r1[e] - s_c[1]) * g.spy, k2 = ((double)r2[e] - s_c[2]) * g.spy;
                const double k3 = ((double)r3[e] - s_c[3]) * g.spy, k4 = ((double)r4[e] - s_c[4]) * g.spy;
                const double v = g.x[e] + s_c[0] * (((k1 + 2 * k2) + 2 * k3) + k4);
                g.x[e] = v;
                if (last) g.w[e] = v;
            }
        }
        if (threadIdx.x == 0) {
            const double tn = s_t + h;
            s_t = tn;   // read after the grid barrier below
            if (lead) {
                ctl->t = tn;
                ctl->n_accept++;
            }
        }
        TRACE();
        if (!grid_barrier(g, bar_target)) return;
        TRACE();
        if (threadIdx.x == 0 && step == 0) s_trk = -1;   // trace the first step only
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

// The same split for the kernel sequence's stage states, which also keeps
// dxw = (xhi - w_ref,hi) + (xlo - w_ref,lo), the state part of the mantle
// term, in the order the step engine's phase A forms it.
__global__ void k_split_dxw(const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo,
                            const float* __restrict__ wrhi, const float* __restrict__ wrlo, float* __restrict__ dxw,
                            size_t n)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const double v = x[e];
        const float a = (float)v;
        const float b = (float)(v - (double)a);
        hi[e] = a;
        lo[e] = b;
        dxw[e] = (a - wrhi[e]) + (b - wrlo[e]);
    }
}

void split_hilo_dxw(const double* x, float* hi, float* lo, const float* wrhi, const float* wrlo, float* dxw, size_t n,
                    cudaStream_t s)
{
    int b = (int)((n + 255) / 256);
    if (b > 1216) b = 1216;
    k_split_dxw<<<b, 256, 0, s>>>(x, hi, lo, wrhi, wrlo, dxw, n);
}

template <typename T, int RA, int FM> int engine_config_shape(const Plan2D& p, int nsm, int optin, int* grid, int* CB,
                                                     size_t* smem)
{
    const int cb = EngShape<RA>::cb;
    *CB = cb;
    *smem = engine_smem_bytes<T, RA>(p, cb);
    if (*smem > (size_t)optin) return 0;
    {
        // the limit is a property of the kernel, shared by every handle:
        // only ever raise it, so a handle of a smaller domain created later
        // does not lower it under a larger one
        static std::mutex mu;
        static size_t cur = 0;
        std::lock_guard<std::mutex> lk(mu);
        if (*smem > cur) {
            if (cudaFuncSetAttribute(k_engine_rk4<T, RA, FM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) !=
                cudaSuccess)
                return 0;
            cur = *smem;
        }
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_engine_rk4<T, RA, FM>, EngShape<RA>::threads, *smem) !=
            cudaSuccess ||
        per_sm < 1)
        return 0;
    if (per_sm > EngShape<RA>::per_sm) per_sm = EngShape<RA>::per_sm;
    // no more blocks than the largest phase has work items: a small domain
    // then leaves SMs free for other handles' work (serving, ensembles)
    const int na = (p.ny + RA - 1) / RA, nb = (p.h + 1 + cb - 1) / cb, nc = na;
    // the stencil phase must fit one wave of resident blocks: beyond that
    // (1024^2) every barrier waits for several items in a row and the kernel
    // sequence is faster (measured 5.4 ms per update in the engine against
    // 13.4 / 4 ms per 1024^2-sized quarter of a 2048^2 update in the kernel
    // sequence)
    if (na > per_sm * nsm) return 0;
    int items = na > nb ? na : nb;
    if (nc > items) items = nc;
    *grid = per_sm * nsm < items ? per_sm * nsm : items;
    return 1;
}

template <typename T> int engine_config(const Plan2D& p, int* grid, int* CB, size_t* smem, int* RA, int* P2)
{
    // The plain FP64 form is FP64-throughput bound; it runs faster as the
    // multi-kernel graph (full occupancy) than in the one-grid engine.
    if (sizeof(T) == 8) return 0;
    int dev = 0, nsm = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // four-row items when there are enough of them for three quarters of the SMs
    int ra = (p.ny + 3) / 4 >= (3 * nsm + 3) / 4 ? 4 : 2;
    // FI_ENGINE_RA: rows per stencil item, 2 or 4 (tuning)
    if (const char* ev = getenv("FI_ENGINE_RA")) {
        const int v = atoi(ev);
        if (v == 2 || v == 4) ra = v;
    }
    const int p2 = ((p.h & (p.h - 1)) == 0 && (p.ny & (p.ny - 1)) == 0) ? 1 : 0;
    *P2 = p2;
    if constexpr (sizeof(T) == 4) {
        auto shape = [&](int r) {
            if (r == 4) return p2 ? engine_config_shape<T, 4, FFT_POW2>(p, nsm, optin, grid, CB, smem)
                                  : engine_config_shape<T, 4, FFT_ANY>(p, nsm, optin, grid, CB, smem);
            return p2 ? engine_config_shape<T, 2, FFT_POW2>(p, nsm, optin, grid, CB, smem)
                      : engine_config_shape<T, 2, FFT_ANY>(p, nsm, optin, grid, CB, smem);
        };
        if (ra == 4 && shape(4)) {
            *RA = 4;
            return 1;
        }
        *RA = 2;
        return shape(2);
    }
    return 0;
}

template <typename T> cudaError_t engine_launch(const EngineArgs& g, int grid, size_t smem, cudaStream_t s)
{
    if constexpr (sizeof(T) == 8) {
        return cudaErrorNotSupported;   // engine_config never selects the plain form
    } else {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(g.ra == 4 ? EngShape<4>::threads : EngShape<2>::threads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if (g.ra == 4) return g.p2 ? cudaLaunchKernelEx(&cfg, k_engine_rk4<T, 4, FFT_POW2>, g)
                                   : cudaLaunchKernelEx(&cfg, k_engine_rk4<T, 4, FFT_ANY>, g);
        return g.p2 ? cudaLaunchKernelEx(&cfg, k_engine_rk4<T, 2, FFT_POW2>, g)
                    : cudaLaunchKernelEx(&cfg, k_engine_rk4<T, 2, FFT_ANY>, g);
    }
}

template int engine_config<float>(const Plan2D&, int*, int*, size_t*, int*, int*);
template int engine_config<double>(const Plan2D&, int*, int*, size_t*, int*, int*);
template cudaError_t engine_launch<float>(const EngineArgs&, int, size_t, cudaStream_t);
template cudaError_t engine_launch<double>(const EngineArgs&, int, size_t, cudaStream_t);

}  // namespace fi
