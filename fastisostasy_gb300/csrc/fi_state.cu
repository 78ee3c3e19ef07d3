// fi_state.cu — sea level, column anomalies, barystatic sums, integrator
// stages and the update tail, all in double precision.
//
// Restates, per cell and fused into few passes:
//   calc_Haf, calc_masks, calc_columnanoms_*, calc_mass_anom, calc_z_ss,
//   calc_sl_contributions                       src/sealevel.f90:25-205
//   the bsl_now update of isos_update           src/fastisostasy.f90:766-777
//   step_euler / step_rk4 / step_tsit54 stages  src/integrators.f90:12-203
//   the update tail + check_isos_instabilities  src/fastisostasy.f90:856-899
// Grid reductions are deterministic: every block reduces its cells in a
// fixed tree, writes one partial, and the last block to arrive combines the
// partials in block order.
#include <cstdio>

#include "fi_batch.h"
#include "fi_state.h"

namespace fi {

constexpr int NT = 256;

// |x| as the bit pattern of a double (sign cleared); above kInfBits it is a NaN
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;
__device__ __forceinline__ unsigned long long abs_bits(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
// m = max(m, |x|) on the bit patterns, NaN ignored as fmax ignores it
__device__ __forceinline__ void absmax_bits(unsigned long long& m, double x)
{
    const unsigned long long b = abs_bits(x);
    if (b <= kInfBits && b > m) m = b;
}

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Reduce NV values per thread across the block (sum or max per slot).
template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], const bool (&is_max)[NV], double* sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = is_max[q] ? warp_max(v[q]) : warp_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[wid * NV + q] = v[q];
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double a = (lane < nw) ? sh[lane * NV + q] : (is_max[q] ? 0.0 : 0.0);
            v[q] = is_max[q] ? warp_max(a) : warp_sum(a);
        }
    }
}

// Block partials -> the last block to arrive combines them: thread t sums
// partials t, t+NT, ... in order, then the same fixed tree as block_reduce.
// The combination order depends only on gridDim, so results are
// run-to-run deterministic.  Returns true in thread 0 of the last block,
// with the totals in `tot`.
template <int NV>
__device__ bool grid_finish(double (&v)[NV], const bool (&is_max)[NV], double* partials, unsigned* counter,
                            double (&tot)[NV], int bid, int nblk)
{
    __shared__ double sh[32 * NV];
    __shared__ bool last;
    block_reduce<NV>(v, is_max, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) partials[(size_t)bid * NV + q] = v[q];
        __threadfence();
        const unsigned prev = atomicAdd(counter, 1u);
        last = (prev == (unsigned)nblk - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double a[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        a[q] = 0.0;
        for (unsigned b = threadIdx.x; b < (unsigned)nblk; b += blockDim.x) {
            const double pb = ((volatile double*)partials)[(size_t)b * NV + q];
            a[q] = is_max[q] ? fmax(a[q], pb) : a[q] + pb;
        }
    }
    __syncthreads();
    block_reduce<NV>(a, is_max, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) tot[q] = a[q];
        *counter = 0u;
        return true;
    }
    return false;
}

// grid_finish with the per-block part in FP32 (this GPU runs FP64 at 1/64
// of the FP32 rate): maxima and sums of the block's threads reduced in
// float, the block totals passed on as doubles and combined as above.
__device__ __forceinline__ float warp_sum_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

template <int NV>
__device__ bool grid_finish_f(float (&vf)[NV], const bool (&is_max)[NV], double* partials, unsigned* counter,
                              double (&tot)[NV], int bid, int nblk)
{
    __shared__ float shf[32 * NV];
    __shared__ double sh[32 * NV];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) vf[q] = is_max[q] ? warp_max_f(vf[q]) : warp_sum_f(vf[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) shf[wid * NV + q] = vf[q];
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const float a = (lane < nw) ? shf[lane * NV + q] : 0.f;
            vf[q] = is_max[q] ? warp_max_f(a) : warp_sum_f(a);
        }
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) partials[(size_t)bid * NV + q] = (double)vf[q];
        __threadfence();
        const unsigned prev = atomicAdd(counter, 1u);
        last = (prev == (unsigned)nblk - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double a[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        a[q] = 0.0;
        for (unsigned b = threadIdx.x; b < (unsigned)nblk; b += blockDim.x) {
            const double pb = ((volatile double*)partials)[(size_t)b * NV + q];
            a[q] = is_max[q] ? fmax(a[q], pb) : a[q] + pb;
        }
    }
    __syncthreads();
    block_reduce<NV>(a, is_max, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) tot[q] = a[q];
        *counter = 0u;
        return true;
    }
    return false;
}

// The same over this launch's grid.
template <int NV>
__device__ __forceinline__ bool grid_finish(double (&v)[NV], const bool (&is_max)[NV], double* partials,
                                            unsigned* counter, double (&tot)[NV])
{
    return grid_finish<NV>(v, is_max, partials, counter, tot, (int)blockIdx.x, (int)gridDim.x);
}

// Scalar work done once per block (FP64 throughput is low on this part):
// the corner mean of a field, broadcast through shared memory.
template <typename T> __device__ __forceinline__ double block_corner_mean(const T* a, int nx, int ny)
{
    __shared__ double s_cm;
    __syncthreads();
    if (threadIdx.x == 0) s_cm = corner_mean_of(a, nx, ny);
    __syncthreads();
    return s_cm;
}

// Per-block scalars of the mixed-form update kernels.  GB300 executes FP64
// instructions, conversions included, at 1/64 of the FP32 rate: a preamble
// of ten FP64 operations in every thread costs more than the few cells each
// thread then updates.  Thread 0 evaluates the scalars (in FP64, as before)
// and the block reads the float results from shared memory.
struct BlockScal {
    float f[6];
    double d;
};
template <typename F> __device__ __forceinline__ BlockScal block_scalars(F&& eval)
{
    __shared__ BlockScal s_bs;
    __syncthreads();
    if (threadIdx.x == 0) s_bs = eval();
    __syncthreads();
    return s_bs;
}

__device__ __forceinline__ bool in_crop(const Dom& d, int i, int j)
{
    return i >= d.i0 && i < d.i0 + d.nxi && j >= d.j0 && j < d.j0 + d.nyi;
}

// --- 1. Hice <- H_ice, Haf, sea-level contribution sums -------------------
__global__ void __launch_bounds__(NT) k_upd_begin(Dom d, const double* __restrict__ H_ice)
{
    double v[2] = {0.0, 0.0};
    const bool mx[2] = {false, false};
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < d.n; e += (size_t)gridDim.x * NT) {
        // 32-bit index arithmetic (a 64-bit division is a long instruction
        // sequence; a padded grid has far fewer than 2^32 cells)
        const unsigned eu = (unsigned)e, nxu = (unsigned)d.nx;
        const unsigned ju = eu / nxu;
        const int j = (int)ju, i = (int)(eu - ju * nxu);
        double H = 0.0;
        if (H_ice && in_crop(d, i, j)) H = H_ice[(size_t)(j - d.j0) * d.nxi + (i - d.i0)];
        else if (!H_ice) H = d.Hice[e];
        d.Hice[e] = H;
        // calc_Haf, src/sealevel.f90:132-145
        double h = (d.z_ss[e] - d.z_bed[e]) * d.rho_sw_over_ice;
        if (h < 0.0) h = 0.0;
        h = H - h;
        if (h < 0.0) h = 0.0;
        d.Haf[e] = h;
        v[0] += (h - d.Haf_ref[e]) * d.A[e];
        v[1] += ((H - d.Hice_ref[e]) * d.Vden) * d.A[e];
    }
    double tot[2];
    if (grid_finish<2>(v, mx, d.partials, &d.ctl->counter[0], tot)) {
        Ctl* c = d.ctl;
        const double V_old = (c->V_af + c->V_den) + c->V_pov;
        c->V_af = tot[0] * d.rho_ice_over_sw;
        c->V_den = tot[1];
        c->V_pov = 0.0;
        c->deltaV = ((c->V_af + c->V_den) + c->V_pov) - V_old;
        // bsl_now update, src/fastisostasy.f90:766-777
        if (c->bsl_method == 2) c->bsl = c->bsl - c->deltaV / c->A_ocean;
        if (c->bsl_method == 3) {
            c->dbsl_total = c->dbsl_total + c->deltaV / c->A_ocean;
            c->bsl = c->bsl - c->dbsl_total;
        }
    }
}

// --- 2. z_ss, masks, ice/seawater/load anomalies (+ elastic conv input) ---
template <typename T>
__global__ void __launch_bounds__(NT) k_upd_masks(Dom d, T* __restrict__ conv_in)
{
    const double bsl = d.ctl->bsl;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < d.n; e += (size_t)gridDim.x * NT) {
        const double zss = (bsl + d.z_ss_ref[e]) + d.dz_ss[e];
        d.z_ss[e] = zss;
        const double Haf = d.Haf[e], H = d.Hice[e];
        const bool cont = d.z_bed[e] > zss;
        const bool grd = (H > 0.0) && (Haf > 0.0);
        const bool ocean = !(cont || grd);
        d.m_cont[e] = cont;
        d.m_grounded[e] = grd;
        d.m_ocean[e] = ocean;
        const double cice = 0.0 + d.rho_ice * (Haf - d.Haf_ref[e]);
        const double csw = 0.0 + (ocean ? d.rho_w * (zss - d.z_ss_ref[e]) : 0.0);
        d.c_ice[e] = cice;
        d.c_sw[e] = csw;
        double cl = cice;
        if (d.interactive) cl = cl + csw;
        cl = d.mactive[e] ? cl : 0.0;
        d.c_load[e] = cl;
        if (conv_in) conv_in[e] = (T)((cl * d.g) * d.K2[e]);
    }
}

// --- 3. elastic displacement, lithosphere/full anomalies, mass (+ geoid input)
// we_mode: 0 keep we, 1 we = we_raw - corner mean, 2 we = 0
template <typename T>
__global__ void __launch_bounds__(NT)
k_upd_litho(Dom d, const double* __restrict__ we_raw, const double* __restrict__ corners, int we_mode,
            T* __restrict__ conv_in)
{
    double cm = 0.0;
    if (we_mode == 1) cm = corner_mean(corners[0], corners[1], corners[2], corners[3]);
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < d.n; e += (size_t)gridDim.x * NT) {
        double we = d.we[e];
        if (we_mode == 1) we = we_raw[e] - cm;
        else if (we_mode == 2) we = 0.0;
        d.we[e] = we;
        const double cli = 0.0 + d.rho_l * (we - d.we_ref[e]);
        d.c_litho[e] = cli;
        const bool act = d.mactive[e];
        const double cf = act ? (d.c_load[e] + cli) + d.c_mantle[e] : 0.0;
        d.c_full[e] = cf;
        const double ma = act ? d.A[e] * cf : 0.0;
        d.mass[e] = ma;
        if (conv_in) conv_in[e] = (T)ma;
    }
}

// --- 4. sea-surface perturbation, z_ss, masks, load; RHS load term q0 ------
// dz_mode: 0 keep, 1 dz_ss = raw - corner mean, 2 dz_ss = 0
// stage_mode 0 (reference): q0 = -g * canom_full (mantle anomaly frozen);
// stage_mode 1 (true stages): q0 = -g * (canom_load + canom_litho).
template <typename T>
__global__ void __launch_bounds__(NT)
k_upd_load(Dom d, const double* __restrict__ dz_raw, const double* __restrict__ corners, int dz_mode,
           T* __restrict__ q0, int stage_mode, int run_integrator)
{
    double cm = 0.0;
    if (dz_mode == 1) cm = corner_mean(corners[0], corners[1], corners[2], corners[3]);
    const double bsl = d.ctl->bsl;
    // get_dwdt refreshes canom_full only if a step runs
    const bool will_step = run_integrator && d.ctl->t < d.ctl->tf;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < d.n; e += (size_t)gridDim.x * NT) {
        double dz = d.dz_ss[e];
        if (dz_mode == 1) dz = dz_raw[e] - cm;
        else if (dz_mode == 2) dz = 0.0;
        d.dz_ss[e] = dz;
        const double zss = (bsl + d.z_ss_ref[e]) + dz;
        d.z_ss[e] = zss;
        const double Haf = d.Haf[e], H = d.Hice[e];
        const bool cont = d.z_bed[e] > zss;
        const bool grd = (H > 0.0) && (Haf > 0.0);
        const bool ocean = !(cont || grd);
        d.m_cont[e] = cont;
        d.m_grounded[e] = grd;
        d.m_ocean[e] = ocean;
        const double csw = 0.0 + (ocean ? d.rho_w * (zss - d.z_ss_ref[e]) : 0.0);
        d.c_sw[e] = csw;
        double cl = d.c_ice[e];
        if (d.interactive) cl = cl + csw;
        const bool act = d.mactive[e];
        cl = act ? cl : 0.0;
        d.c_load[e] = cl;
        if (stage_mode == 0) {
            const double cf = act ? (cl + d.c_litho[e]) + d.c_mantle[e] : 0.0;
            if (will_step) d.c_full[e] = cf;
            q0[e] = (T)(act ? -d.g * cf : 0.0);
        } else {
            q0[e] = (T)(act ? -d.g * (cl + d.c_litho[e]) : 0.0);
        }
    }
}

// --- per-update arguments ----------------------------------------------------
// Target time and barystatic scalars of one isos_update, written by a kernel
// so that the host never waits and a captured update graph reads them from
// the control block.
__device__ __forceinline__ void set_args_one(Ctl* c, double tf, double bsl, double A_ocean, int method,
                                             int write_bsl)
{
    c->tf = tf;
    c->rej0 = c->n_reject;
    if (write_bsl) c->bsl = bsl;
    c->A_ocean = A_ocean;
    c->bsl_method = method;
}

__global__ void k_set_args(Ctl* c, double tf, double bsl, double A_ocean, int method, int write_bsl)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    set_args_one(c, tf, bsl, A_ocean, method, write_bsl);
}

// --- integrator control ------------------------------------------------------
// kind 0 euler (clips ode%dt), 1 rk4 (local h), 2 tsit54 (clips ode%dt)
__global__ void k_step_begin(Ctl* c, int kind)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double tf = c->tf;
    if (c->status != ST_OK || !(c->t < tf)) { c->done = 1; return; }
    c->done = 0;
    if (kind == 1) c->h = fmin(c->dt, tf - c->t);
    else { c->dt = fmin(c->dt, tf - c->t); c->h = c->dt; }
}

// y = x + (a*h) * k,  k = (raw - corner_mean(raw)) * spy.
// Plain form: double throughout.  Mixed form: the increment is formed in
// float and added to the double state (one double add per cell).
template <typename T>
__global__ void __launch_bounds__(NT)
k_rk_stage(const Ctl* __restrict__ c, double* __restrict__ y, const double* __restrict__ x, const T* __restrict__ raw,
           double a, int nx, int ny, double spy)
{
    if (c->done) return;
    const size_t n = (size_t)nx * ny;
    if (sizeof(T) == 8) {
        const double cm = c->plain ? 0.0 : block_corner_mean(raw, nx, ny);
        const double ah = a * c->h;
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
            const double k = ((double)raw[e] - cm) * spy;
            y[e] = x[e] + ah * k;
        }
    } else {
        const BlockScal bs = block_scalars([&] {
            BlockScal r;
            r.f[0] = c->plain ? 0.f : (float)corner_mean_of(raw, nx, ny);
            r.f[1] = (float)((a * c->h) * spy);
            return r;
        });
        const float cmf = bs.f[0], sc = bs.f[1];
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
            y[e] = x[e] + (double)(((float)raw[e] - cmf) * sc);
    }
}

// RK4 combination x += (h/6)*(k1 + 2k2 + 2k3 + k4), w = x.
// Reference mode passes the same raw four times (get_dwdt ignores its state).
template <typename T>
__global__ void __launch_bounds__(NT)
k_rk4_final(Ctl* c, double* __restrict__ x, double* __restrict__ w, const T* __restrict__ r1,
            const T* __restrict__ r2, const T* __restrict__ r3, const T* __restrict__ r4, int nx, int ny,
            double spy)
{
    if (c->done) return;
    __shared__ double s[5];
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool pl = c->plain != 0;
        s[0] = c->h / 6;
        s[1] = pl ? 0.0 : corner_mean_of(r1, nx, ny);
        s[2] = pl ? 0.0 : corner_mean_of(r2, nx, ny);
        s[3] = pl ? 0.0 : corner_mean_of(r3, nx, ny);
        s[4] = pl ? 0.0 : corner_mean_of(r4, nx, ny);
    }
    __syncthreads();
    const double h6 = s[0], c1 = s[1], c2 = s[2], c3 = s[3], c4 = s[4];
    const size_t n = (size_t)nx * ny;
    if (sizeof(T) == 8) {
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
            const double k1 = ((double)r1[e] - c1) * spy, k2 = ((double)r2[e] - c2) * spy;
            const double k3 = ((double)r3[e] - c3) * spy, k4 = ((double)r4[e] - c4) * spy;
            const double v = x[e] + h6 * (((k1 + 2 * k2) + 2 * k3) + k4);
            x[e] = v;
            w[e] = v;
        }
    } else {
        const BlockScal bs = block_scalars([&] {
            BlockScal r;
            r.f[0] = (float)c1; r.f[1] = (float)c2; r.f[2] = (float)c3; r.f[3] = (float)c4;
            r.f[4] = (float)(h6 * spy);
            return r;
        });
        const float f1 = bs.f[0], f2 = bs.f[1], f3 = bs.f[2], f4 = bs.f[3], sc = bs.f[4];
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
            const float k = ((((float)r1[e] - f1) + 2.f * ((float)r2[e] - f2)) + 2.f * ((float)r3[e] - f3)) +
                            ((float)r4[e] - f4);
            const double v = x[e] + (double)(k * sc);
            x[e] = v;
            w[e] = v;
        }
    }
}

// Mixed RK4 combination that also carries the float pair of x (the stage
// RHS of the next step reads x as xhi + xlo): the FP64 state takes the float
// increment, the pair the same increment by an FP32 two-sum, as in the step
// engine's state update; dxw = (xhi - w_ref,hi) + (xlo - w_ref,lo) of the new
// pair feeds the mantle term of the next step's stages.
__global__ void __launch_bounds__(NT)
k_rk4_final_pair(Ctl* c, double* __restrict__ x, double* __restrict__ w, float* __restrict__ xhi,
                 float* __restrict__ xlo, const float* __restrict__ wrhi, const float* __restrict__ wrlo,
                 float* __restrict__ dxw, const float* __restrict__ r1, const float* __restrict__ r2,
                 const float* __restrict__ r3, const float* __restrict__ r4, int nx, int ny, double spy)
{
    if (c->done) return;
    const BlockScal bs = block_scalars([&] {
        BlockScal r;
        r.f[0] = (float)corner_mean_of(r1, nx, ny);
        r.f[1] = (float)corner_mean_of(r2, nx, ny);
        r.f[2] = (float)corner_mean_of(r3, nx, ny);
        r.f[3] = (float)corner_mean_of(r4, nx, ny);
        r.f[4] = (float)((c->h / 6) * spy);
        return r;
    });
    const float f1 = bs.f[0], f2 = bs.f[1], f3 = bs.f[2], f4 = bs.f[3], sc = bs.f[4];
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
        const float k = ((((float)r1[e] - f1) + 2.f * ((float)r2[e] - f2)) + 2.f * ((float)r3[e] - f3)) +
                        ((float)r4[e] - f4);
        const float inc = k * sc;
        const double v = x[e] + (double)inc;
        x[e] = v;
        w[e] = v;
        const float hi = xhi[e], lo = xlo[e];
        const float sm = hi + inc, bb = sm - hi;
        const float er = (hi - (sm - bb)) + (inc - bb);
        const float l2 = lo + er;
        const float h2 = sm + l2;
        const float lo2 = l2 - (h2 - sm);
        xhi[e] = h2;
        xlo[e] = lo2;
        dxw[e] = (h2 - wrhi[e]) + (lo2 - wrlo[e]);
    }
}

__global__ void k_step_end(Ctl* c)
{
    if (threadIdx.x != 0 || blockIdx.x != 0 || c->done) return;
    c->t = c->t + c->h;
    c->n_accept++;
}

// Euler: x += dt*k, w = x
template <typename T>
__global__ void __launch_bounds__(NT)
k_euler_final(const Ctl* __restrict__ c, double* __restrict__ x, double* __restrict__ w, const T* __restrict__ r1,
              int nx, int ny, double spy)
{
    if (c->done) return;
    const size_t n = (size_t)nx * ny;
    if (sizeof(T) == 8) {
        const double c1 = c->plain ? 0.0 : block_corner_mean(r1, nx, ny);
        const double h = c->h;
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
            const double v = x[e] + h * (((double)r1[e] - c1) * spy);
            x[e] = v;
            w[e] = v;
        }
    } else {
        const BlockScal bs = block_scalars([&] {
            BlockScal r;
            r.f[0] = c->plain ? 0.f : (float)corner_mean_of(r1, nx, ny);
            r.f[1] = (float)(c->h * spy);
            return r;
        });
        const float f1 = bs.f[0], sc = bs.f[1];
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
            const double v = x[e] + (double)(((float)r1[e] - f1) * sc);
            x[e] = v;
            w[e] = v;
        }
    }
}

// --- Tsitouras 5(4), reference-compatible (single distinct RHS value) --------
__constant__ double c_ts_b[6] = {0.0845, 0.0, 0.0, 0.5179, 0.1276, 0.2700};
__constant__ double c_ts_bh[6] = {0.0845, 0.0, 0.0, 0.5179, 0.1276, 0.2700 - 1 / 5.0};

__device__ __forceinline__ void ts_x12(double x, double k, double dt, double& x1, double& x2)
{
    // x1 = x + sum_s (dt bh_s) k and x2 = x + sum_s (dt b_s) k in the
    // reference's order.  b_1 = b_2 = 0 (those terms add an exact zero) and
    // bh_s = b_s for s < 5, so both sums share their first three terms.
    double a = x;
    a = a + (dt * c_ts_b[0]) * k;
    a = a + (dt * c_ts_b[3]) * k;
    a = a + (dt * c_ts_b[4]) * k;
    x1 = a + (dt * c_ts_bh[5]) * k;
    x2 = a + (dt * c_ts_b[5]) * k;
}

// Accept or reject an attempt from its error norm, adapt dt
// (src/integrators.f90:186-199, tsit54 step control).  The reference halves
// dt without a floor and never reads dt_min; here a rejection that takes dt
// below dt_min, or one past the per-update rejection limit, ends the update
// with ST_STEP (FI_E_STEP on the host).
__device__ __forceinline__ void ts_decide(Ctl* c, double err, double dt, double q, double dt_max)
{
    c->err = err;
    c->n_attempt++;
    if (err < 1) {
        c->accepted = 1;
        c->t = c->t + dt;
        c->dt = fmin(dt * pow(1 / err, 1 / q), dt_max);
        c->n_accept++;
    } else {
        c->accepted = 0;
        c->dt = dt * 0.5;
        c->n_reject++;
        if (c->n_reject - c->rej0 > c->max_reject || c->dt < c->dt_min) { c->status = ST_STEP; c->done = 1; }
    }
}

template <typename T>
__device__ __forceinline__ void ts_max_body(Dom d, const T* __restrict__ raw, double atol, double rtol, int bid, int nblk)
{
    Ctl* c = d.ctl;
    if (c->done) return;
    const double dt = c->h;
    const double cm = c->plain ? 0.0 : block_corner_mean(raw, d.nx, d.ny);
    double v[2] = {0.0, 0.0};
    const bool mx[2] = {true, true};
    if constexpr (sizeof(T) == 4) {
        // mixed form: k, the error term x2 - x1 = dt (b_5 - bh_5) k and the
        // magnitudes for the tolerance in FP32; only the state update
        // x2 = x + dt (sum_s b_s) k stays in FP64
        const double cx = ((dt * c_ts_b[0] + dt * c_ts_b[3]) + dt * c_ts_b[4]) + dt * c_ts_b[5];
        const float ce = (float)(dt * c_ts_b[5] - dt * c_ts_bh[5]);
        const float cmf = (float)cm, spyf = (float)d.spy;
        float m1 = 0.f, m2 = 0.f;
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            const float k = ((float)raw[e] - cmf) * spyf;
            const double x2 = d.x[e] + cx * (double)k;
            const float dx = ce * k;
            d.ts_x2[e] = x2;
            ((float*)d.ts_dx)[e] = dx;
            const float x2f = (float)x2;
            m1 = fmaxf(m1, fabsf(x2f - dx));
            m2 = fmaxf(m2, fabsf(x2f));
        }
        v[0] = (double)m1;
        v[1] = (double)m2;
    } else {
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            const double k = ((double)raw[e] - cm) * d.spy;
            double x1, x2;
            ts_x12(d.x[e], k, dt, x1, x2);
            d.ts_x2[e] = x2;         // kept for the error norm and the commit
            d.ts_dx[e] = x2 - x1;
            v[0] = fmax(v[0], fabs(x1));
            v[1] = fmax(v[1], fabs(x2));
        }
    }
    double tot[2];
    if (grid_finish<2>(v, mx, d.partials, &c->counter[1], tot, bid, nblk)) c->tol = atol + rtol * fmax(tot[0], tot[1]);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_ts_max(Dom d, const T* __restrict__ raw, double atol, double rtol)
{
    ts_max_body<T>(d, raw, atol, rtol, (int)blockIdx.x, (int)gridDim.x);
}

template <typename T>
__device__ __forceinline__ void ts_err_body(Dom d, const T* __restrict__ raw, double q, double dt_max, int bid, int nblk)
{
    Ctl* c = d.ctl;
    if (c->done) return;
    const double dt = c->h, inv_tol = 1.0 / c->tol;
    double v[1] = {0.0};
    const bool mx[1] = {false};
    if constexpr (sizeof(T) == 4) {
        const float it = (float)inv_tol;
        float acc = 0.f;
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            const float r = ((const float*)d.ts_dx)[e] * it;   // (x2 - x1) / tol
            acc += r * r;
        }
        v[0] = (double)acc;
    } else {
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            const double r = d.ts_dx[e] * inv_tol;   // (x2 - x1) / tol
            v[0] += r * r;
        }
    }
    double tot[1];
    if (grid_finish<1>(v, mx, d.partials, &c->counter[2], tot, bid, nblk)) ts_decide(c, sqrt(tot[0] / (double)d.n), dt, q, dt_max);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_ts_err(Dom d, const T* __restrict__ raw, double q, double dt_max)
{
    ts_err_body<T>(d, raw, q, dt_max, (int)blockIdx.x, (int)gridDim.x);
}

// Mixed form with now%w as a float pair (whi + wlo), one pass per attempt:
// k, the error term dx = x2 - x1 = dt (b_5 - bh_5) k, x2 in FP32 from the
// pair for the tolerance magnitudes, and sum dx^2 reduced with them; the
// last block sets tol = atol + rtol max(|x1|, |x2|) and err = sqrt(sum dx^2
// / n) / tol, which is the reference's sqrt(sum ((x2 - x1) / tol)^2 / n)
// with the constant 1/tol taken out of the sum, and decides.  No FP64 work
// per cell here: the FP64 state update moves to ts_commit_pair_body, which
// runs for accepted attempts only.
__device__ __forceinline__ void ts_fused_body(Dom d, const float* __restrict__ raw, double atol, double rtol, double q,
                                              double dt_max, int bid, int nblk)
{
    Ctl* c = d.ctl;
    if (c->done) return;
    const double dt = c->h;
    const BlockScal bs = block_scalars([&] {
        BlockScal r;
        r.f[0] = (float)(((dt * c_ts_b[0] + dt * c_ts_b[3]) + dt * c_ts_b[4]) + dt * c_ts_b[5]);
        r.f[1] = (float)(dt * c_ts_b[5] - dt * c_ts_bh[5]);
        r.f[2] = c->plain ? 0.f : (float)corner_mean_of(raw, d.nx, d.ny);
        r.f[3] = (float)d.spy;
        return r;
    });
    const float cxf = bs.f[0], ce = bs.f[1], cmf = bs.f[2], spyf = bs.f[3];
    float m1 = 0.f, m2 = 0.f, s2 = 0.f;
    // unrolled so that several cells' loads are in flight per thread
#pragma unroll 4
    for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
        const float k = (raw[e] - cmf) * spyf;
        const float dx = ce * k;
        const float x2f = d.whi[e] + (d.wlo[e] + cxf * k);
        m1 = fmaxf(m1, fabsf(x2f - dx));
        m2 = fmaxf(m2, fabsf(x2f));
        s2 += dx * dx;
    }
    float v[3] = {m1, m2, s2};
    const bool mx[3] = {true, true, false};
    double tot[3];
    if (grid_finish_f<3>(v, mx, d.partials, &c->counter[1], tot, bid, nblk)) {
        const double tol = atol + rtol * fmax(tot[0], tot[1]);
        c->tol = tol;
        ts_decide(c, sqrt(tot[2] / (double)d.n) / tol, dt, q, dt_max);
    }
}

// Accepted attempt of the fused mixed form: x = x + dt (sum_s b_s) k in
// FP64 (k as ts_max_body forms it), now%w = x, and the float pair takes the
// same increment by an FP32 two-sum.
__device__ __forceinline__ void ts_commit_pair_body(Dom d, const float* __restrict__ raw, int bid, int nblk)
{
    const Ctl* c = d.ctl;
    if (c->done || !c->accepted) return;
    const BlockScal bs = block_scalars([&] {
        const double dt = c->h;
        BlockScal r;
        r.d = ((dt * c_ts_b[0] + dt * c_ts_b[3]) + dt * c_ts_b[4]) + dt * c_ts_b[5];
        r.f[0] = (float)r.d;
        r.f[1] = c->plain ? 0.f : (float)corner_mean_of(raw, d.nx, d.ny);
        r.f[2] = (float)d.spy;
        return r;
    });
    const double cx = bs.d;
    const float cxf = bs.f[0], cmf = bs.f[1], spyf = bs.f[2];
#pragma unroll 4
    for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
        const float k = (raw[e] - cmf) * spyf;
        const double x2 = d.x[e] + cx * (double)k;
        d.x[e] = x2;
        d.w[e] = x2;
        const float inc = cxf * k;
        const float hi = d.whi[e], lo = d.wlo[e];
        const float sm = hi + inc, bb = sm - hi;
        const float er = (hi - (sm - bb)) + (inc - bb);
        const float l2 = lo + er;
        const float h2 = sm + l2;
        d.whi[e] = h2;
        d.wlo[e] = l2 - (h2 - sm);
    }
}

__global__ void __launch_bounds__(NT) k_ts_fused(Dom d, const float* __restrict__ raw, double atol, double rtol,
                                                 double q, double dt_max)
{
    ts_fused_body(d, raw, atol, rtol, q, dt_max, (int)blockIdx.x, (int)gridDim.x);
}

__global__ void __launch_bounds__(NT) k_ts_commit_pair(Dom d, const float* __restrict__ raw)
{
    ts_commit_pair_body(d, raw, (int)blockIdx.x, (int)gridDim.x);
}

// Device-side attempt loop of the reference-compatible Tsit5: the attempts
// of one update run as the body of a CUDA graph WHILE node, so the host never
// waits on an accept/reject decision.  The body is
//   k_ts_attempt_begin, [RHS kernels gated by need_rhs], ts_max, ts_err,
//   ts_commit, k_ts_attempt_end
// and makes the same decisions, in the same order, as the host loop.
__global__ void k_ts_loop_begin(Ctl* c)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    c->rhs_valid = 0;
    c->have_rhs = 0;
    c->loop_iter = 0;
    c->need_rhs = 0;
}

__device__ __forceinline__ void attempt_begin_one(Ctl* c, int max_iter)
{
    const double tf = c->tf;
    if (c->status != ST_OK || !(c->t < tf)) { c->done = 1; c->need_rhs = 0; c->active = 0; return; }
    if (++c->loop_iter > max_iter) {
        c->status = ST_STEP;
        c->done = 1;
        c->need_rhs = 0;
        c->active = 0;
        return;
    }
    c->done = 0;
    c->active = 1;
    c->dt = fmin(c->dt, tf - c->t);
    c->h = c->dt;
    c->need_rhs = c->rhs_valid ? 0 : 1;
    if (c->need_rhs) { c->have_rhs = 1; c->rhs_valid = 1; }
}

__global__ void k_ts_attempt_begin(Ctl* c, int max_iter)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    attempt_begin_one(c, max_iter);
}

// 1 while the member has attempts left.  fsal: the first stage of the next
// attempt is the last stage of an accepted one (true stages), so the
// cached RHS stays valid.
__device__ __forceinline__ int attempt_end_one(Ctl* c, int fsal = 0)
{
    if (!fsal && !c->done && c->accepted) c->rhs_valid = 0;   // the state moved: the next attempt needs a new RHS
    return (!c->done && c->status == ST_OK && c->t < c->tf) ? 1 : 0;
}

// more_out == NULL: sets the WHILE condition `loop`; else writes it there
__global__ void k_ts_attempt_end(Ctl* c, cudaGraphConditionalHandle loop, int fsal, int* more_out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int more = attempt_end_one(c, fsal);
    if (more_out) *more_out = more;
    else cudaGraphSetConditional(loop, more ? 1u : 0u);
}

// --- Tsitouras 5(4) with true stages: the Dormand-Prince 5(4) pair whose
// truncated coefficients the reference prints, with FSAL ----------------------
__constant__ double c_dp_a[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0},
    {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
__constant__ double c_dp_bs[7] = {5179.0 / 57600, 0, 7571.0 / 16695, 393.0 / 640, -92097.0 / 339200, 187.0 / 2100,
                                  1.0 / 40};

// block corner means of the stage outputs 0..ns-1 (shared, one thread each)
template <typename T>
__device__ __forceinline__ void dp_corner_means(const Ctl* c, const DPRaw<T>& r, int ns, int nx, int ny, double* cm)
{
    __syncthreads();
    if (threadIdx.x < (unsigned)ns) cm[threadIdx.x] = c->plain ? 0.0 : corner_mean_of(r.p[threadIdx.x], nx, ny);
    __syncthreads();
}

// Stage state y = x + h sum_{r<i} a_{i r} k_r (i = 1..6; stage 6 is x2).
template <typename T>
__device__ __forceinline__ void dp_stage_body(const Ctl* __restrict__ c, double* __restrict__ y,
                                              const double* __restrict__ x, const DPRaw<T>& r, int i, int nx, int ny,
                                              double spy, int bid, int nblk)
{
    if (c->done) return;
    __shared__ double cm[7];
    dp_corner_means(c, r, i, nx, ny, cm);
    const double h = c->h;
    const size_t n = (size_t)nx * ny;
    if constexpr (sizeof(T) == 8) {
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < n; e += (size_t)nblk * NT) {
            double a = 0.0;
            for (int q = 0; q < i; ++q) a += c_dp_a[i][q] * (((double)r.p[q][e] - cm[q]) * spy);
            y[e] = x[e] + h * a;
        }
    } else {
        // the float coefficients, one thread each (no FP64 preamble in every thread)
        __shared__ float af[6], cmf[6];
        if (threadIdx.x < (unsigned)i) {
            af[threadIdx.x] = (float)(c_dp_a[i][threadIdx.x] * h * spy);
            cmf[threadIdx.x] = (float)cm[threadIdx.x];
        }
        __syncthreads();
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < n; e += (size_t)nblk * NT) {
            float a = 0.f;
            for (int q = 0; q < i; ++q) a += af[q] * ((float)r.p[q][e] - cmf[q]);
            y[e] = x[e] + (double)a;
        }
    }
}

// The same stage state in the mixed form as a float pair: the FP32
// increment a of dp_stage_body added to the pair of x by an FP32 two-sum,
// and dxw = (yhi - w_ref,hi) + (ylo - w_ref,lo), the state part of the
// mantle term, so that the stencil takes no FP64 stage state; stage 6 (x2)
// also in FP64 (x2 non-null) for the error estimate and the commit, the
// same value dp_stage_body writes.
__device__ __forceinline__ void dp_stage_pair_body(const Ctl* __restrict__ c, const float* __restrict__ xhi,
                                                   const float* __restrict__ xlo, const float* __restrict__ wrhi,
                                                   const float* __restrict__ wrlo, float* __restrict__ yhi,
                                                   float* __restrict__ ylo, float* __restrict__ ydw,
                                                   double* __restrict__ x2, const double* __restrict__ x,
                                                   const DPRaw<float>& r, int i, int nx, int ny, double spy, int bid,
                                                   int nblk)
{
    if (c->done) return;
    __shared__ double cm[7];
    dp_corner_means(c, r, i, nx, ny, cm);
    const double h = c->h;
    __shared__ float af[6], cmf[6];
    if (threadIdx.x < (unsigned)i) {
        af[threadIdx.x] = (float)(c_dp_a[i][threadIdx.x] * h * spy);
        cmf[threadIdx.x] = (float)cm[threadIdx.x];
    }
    __syncthreads();
    const size_t n = (size_t)nx * ny;
    // read-only loads (the stage outputs come through a pointer array the
    // compiler cannot tell apart from the stores) and several cells per
    // thread in flight
#pragma unroll 4
    for (size_t e = (size_t)bid * NT + threadIdx.x; e < n; e += (size_t)nblk * NT) {
        float a = 0.f;
        for (int q = 0; q < i; ++q) a += af[q] * (__ldg(r.p[q] + e) - cmf[q]);
        if (x2) x2[e] = __ldg(x + e) + (double)a;
        const float hi = __ldg(xhi + e), lo = __ldg(xlo + e);
        const float sm = hi + a, bb = sm - hi;
        const float er = (hi - (sm - bb)) + (a - bb);
        const float l2 = lo + er;
        const float h2 = sm + l2;
        const float lo2 = l2 - (h2 - sm);
        yhi[e] = h2;
        ylo[e] = lo2;
        ydw[e] = (h2 - __ldg(wrhi + e)) + (lo2 - __ldg(wrlo + e));
    }
}

__global__ void __launch_bounds__(NT)
k_dp_stage_pair(const Ctl* __restrict__ c, const float* __restrict__ xhi, const float* __restrict__ xlo,
                const float* __restrict__ wrhi, const float* __restrict__ wrlo, float* __restrict__ yhi,
                float* __restrict__ ylo, float* __restrict__ ydw, double* __restrict__ x2,
                const double* __restrict__ x, DPRaw<float> r, int i, int nx, int ny, double spy)
{
    dp_stage_pair_body(c, xhi, xlo, wrhi, wrlo, yhi, ylo, ydw, x2, x, r, i, nx, ny, spy, (int)blockIdx.x,
                       (int)gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(NT)
k_dp_stage(const Ctl* __restrict__ c, double* __restrict__ y, const double* __restrict__ x, DPRaw<T> r, int i, int nx,
           int ny, double spy)
{
    dp_stage_body<T>(c, y, x, r, i, nx, ny, spy, (int)blockIdx.x, (int)gridDim.x);
}

// x1 = x + h sum_r bs_r k_r; x2 (stage 6 state) is in ts_x2: store x2 - x1
// and reduce max|x1|, max|x2| into the tolerance.
template <typename T>
__device__ __forceinline__ void dp_err_body(Dom d, const DPRaw<T>& r, double atol, double rtol, int bid, int nblk)
{
    Ctl* c = d.ctl;
    if (c->done) return;
    __shared__ double cm[7];
    dp_corner_means(c, r, 7, d.nx, d.ny, cm);
    const double h = c->h;
    double v[2] = {0.0, 0.0};
    const bool mx[2] = {true, true};
    if constexpr (sizeof(T) == 8) {
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            double a = 0.0;
            for (int q = 0; q < 7; ++q) a += c_dp_bs[q] * (((double)r.p[q][e] - cm[q]) * d.spy);
            const double x1 = d.x[e] + h * a, x2 = d.ts_x2[e];
            d.ts_dx[e] = x2 - x1;
            v[0] = fmax(v[0], fabs(x1));
            v[1] = fmax(v[1], fabs(x2));
        }
    } else {
        // x2 - x1 = h sum_r (a_{6 r} - bs_r) k_r in FP32; the float
        // coefficients one thread each
        __shared__ float ce[7], cmf[7];
        if (threadIdx.x < 7u) {
            const int q = (int)threadIdx.x;
            ce[q] = (float)(((q < 6 ? c_dp_a[6][q] : 0.0) - c_dp_bs[q]) * h * d.spy);
            cmf[q] = (float)cm[q];
        }
        __syncthreads();
        float m1 = 0.f, m2 = 0.f;
#pragma unroll 4
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            float dx = 0.f;
            for (int q = 0; q < 7; ++q) dx += ce[q] * ((float)__ldg(r.p[q] + e) - cmf[q]);
            ((float*)d.ts_dx)[e] = dx;
            const float x2f = (float)__ldg(d.ts_x2 + e);
            m1 = fmaxf(m1, fabsf(x2f - dx));
            m2 = fmaxf(m2, fabsf(x2f));
        }
        v[0] = (double)m1;
        v[1] = (double)m2;
    }
    double tot[2];
    if (grid_finish<2>(v, mx, d.partials, &c->counter[1], tot, bid, nblk)) c->tol = atol + rtol * fmax(tot[0], tot[1]);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_dp_err(Dom d, DPRaw<T> r, double atol, double rtol)
{
    dp_err_body<T>(d, r, atol, rtol, (int)blockIdx.x, (int)gridDim.x);
}

// accepted: the last stage's RHS becomes the next attempt's first (FSAL)
template <typename T>
__global__ void __launch_bounds__(NT) k_fsal_copy(const Ctl* __restrict__ c, T* __restrict__ k0,
                                                  const T* __restrict__ k6, size_t n)
{
    if (c->done || !c->accepted) return;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) k0[e] = k6[e];
}

template <typename T>
__device__ __forceinline__ void ts_commit_body(Dom d, const T* __restrict__ raw, int bid, int nblk)
{
    const Ctl* c = d.ctl;
    if (c->done || !c->accepted) return;
    if (sizeof(T) == 4 && d.whi) {
        // mixed form: now%w's float pair takes the same increment
        // dt (sum_s b_s) k by an FP32 two-sum (no FP64 work per cell)
        const double dt = c->h;
        const float cx = (float)(((dt * c_ts_b[0] + dt * c_ts_b[3]) + dt * c_ts_b[4]) + dt * c_ts_b[5]);
        const float cmf = c->plain ? 0.f : (float)block_corner_mean(raw, d.nx, d.ny), spyf = (float)d.spy;
        for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
            const double x2 = d.ts_x2[e];
            d.x[e] = x2;
            d.w[e] = x2;
            const float inc = cx * (((float)raw[e] - cmf) * spyf);
            const float hi = d.whi[e], lo = d.wlo[e];
            const float sm = hi + inc, bb = sm - hi;
            const float er = (hi - (sm - bb)) + (inc - bb);
            const float l2 = lo + er;
            const float h2 = sm + l2;
            d.whi[e] = h2;
            d.wlo[e] = l2 - (h2 - sm);
        }
        return;
    }
    for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
        const double x2 = d.ts_x2[e];
        d.x[e] = x2;
        d.w[e] = x2;
    }
}

// Accepted attempt of the true-stage Tsit5 in the mixed form: x = x2 (FP64),
// now%w = x, and the float pair of x with its dxw take those of the stage-6
// state (the pair buffers still hold them).
__device__ __forceinline__ void ts_commit_tpair_body(Dom d, float* __restrict__ xhi, float* __restrict__ xlo,
                                                     float* __restrict__ xdw, const float* __restrict__ yhi,
                                                     const float* __restrict__ ylo, const float* __restrict__ ydw,
                                                     int bid, int nblk)
{
    const Ctl* c = d.ctl;
    if (c->done || !c->accepted) return;
#pragma unroll 4
    for (size_t e = (size_t)bid * NT + threadIdx.x; e < d.n; e += (size_t)nblk * NT) {
        const double x2 = __ldg(d.ts_x2 + e);
        d.x[e] = x2;
        d.w[e] = x2;
        xhi[e] = __ldg(yhi + e);
        xlo[e] = __ldg(ylo + e);
        xdw[e] = __ldg(ydw + e);
    }
}

__global__ void __launch_bounds__(NT)
k_ts_commit_tpair(Dom d, float* __restrict__ xhi, float* __restrict__ xlo, float* __restrict__ xdw,
                  const float* __restrict__ yhi, const float* __restrict__ ylo, const float* __restrict__ ydw)
{
    ts_commit_tpair_body(d, xhi, xlo, xdw, yhi, ylo, ydw, (int)blockIdx.x, (int)gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_ts_commit(Dom d, const T* __restrict__ raw)
{
    ts_commit_body<T>(d, raw, (int)blockIdx.x, (int)gridDim.x);
}

// --- update tail -----------------------------------------------------------
// w -= corner mean (apply_zerobc_at_corners), canom_mantle, z_bed, dwdt output,
// instability and NaN checks (src/fastisostasy.f90:856-869, :874-899).
template <typename T>
__global__ void __launch_bounds__(NT) k_upd_end(Dom d, const T* __restrict__ raw_last, int have_rhs_arg)
{
    // have_rhs_arg < 0: the update ran the device Tsit5 loop, which recorded it
    const int have_rhs = have_rhs_arg >= 0 ? have_rhs_arg : d.ctl->have_rhs;
    __shared__ double s_c[2];
    if (threadIdx.x == 0) {
        s_c[0] = corner_mean_of(d.w, d.nx, d.ny);
        s_c[1] = (have_rhs && !d.ctl->plain) ? corner_mean_of(raw_last, d.nx, d.ny) : 0.0;
    }
    __syncthreads();
    const double cw = s_c[0], cr = s_c[1];
    // max |w|, |we|, |dz_ss| over the non-NaN cells, on the bit patterns
    // (for non-negative doubles the IEEE order is the integer order of the
    // bits; the FP64 unit is left to the arithmetic), and a NaN flag of z_bed
    unsigned long long m[3] = {0ull, 0ull, 0ull};
    bool nan = false;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < d.n; e += (size_t)gridDim.x * NT) {
        const double w = d.w[e] - cw;
        d.wout[e] = w;
        d.c_mantle[e] = 0.0 + d.rho_m * (w - d.w_ref[e]);
        const double we = d.we[e];
        const double zb = (d.z_bed_ref[e] + w) + we;
        d.z_bed[e] = zb;
        if (have_rhs) d.dwdt[e] = ((double)raw_last[e] - cr) * d.spy;
        absmax_bits(m[0], w);
        absmax_bits(m[1], we);
        absmax_bits(m[2], d.dz_ss[e]);
        nan |= abs_bits(zb) > kInfBits;
    }
    double v[4] = {__longlong_as_double((long long)m[0]), __longlong_as_double((long long)m[1]),
                   __longlong_as_double((long long)m[2]), nan ? 1.0 : 0.0};
    const bool mx[4] = {true, true, true, true};
    double tot[4];
    if (grid_finish<4>(v, mx, d.partials, &d.ctl->counter[3], tot)) {
        Ctl* c = d.ctl;
        c->red[0] = tot[0]; c->red[1] = tot[1]; c->red[2] = tot[2];
        if (c->status == ST_OK) {
            if (tot[0] > 1e5 || tot[1] > 1e5 || tot[2] > 1e3) c->status = ST_LARGE;
            if (tot[3] != 0.0) c->status = ST_NAN;
        }
    }
}

// w was written to d.wout (a separate buffer) so that every block read the
// uncorrected corners; copy it back.
__global__ void __launch_bounds__(NT) k_copy(double* __restrict__ dst, const double* __restrict__ src, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) dst[e] = src[e];
}

// Gather cropped outputs (cropstate2out, src/isos_utils.f90:386-405) into a
// packed buffer: nf fields of nxi*nyi doubles.
__global__ void __launch_bounds__(NT)
k_gather(const double* const* __restrict__ src, const uint8_t* const* __restrict__ msrc, int nf, int nm, Dom d,
         double* __restrict__ out)
{
    const size_t nc = (size_t)d.nxi * d.nyi;
    const size_t tot = nc * (nf + nm);
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < tot; e += (size_t)gridDim.x * NT) {
        const int f = (int)(e / nc);
        const size_t r = e - (size_t)f * nc;
        const int i = (int)(r % d.nxi), j = (int)(r / d.nxi);
        const size_t g = (size_t)(j + d.j0) * d.nx + (i + d.i0);
        out[e] = f < nf ? src[f][g] : (double)msrc[f - nf][g];
    }
}

// The same crop with the masks kept as bytes: nf double fields into out, nm
// byte masks into mout (fi_update's host copy, a quarter fewer bytes).
__global__ void __launch_bounds__(NT)
k_gather_bytes(const double* const* __restrict__ src, const uint8_t* const* __restrict__ msrc, int nf, int nm, Dom d,
               double* __restrict__ out, uint8_t* __restrict__ mout)
{
    const size_t nc = (size_t)d.nxi * d.nyi;
    const size_t tot = nc * (nf + nm);
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < tot; e += (size_t)gridDim.x * NT) {
        const int f = (int)(e / nc);
        const size_t r = e - (size_t)f * nc;
        const int i = (int)(r % d.nxi), j = (int)(r / d.nxi);
        const size_t g = (size_t)(j + d.j0) * d.nx + (i + d.i0);
        if (f < nf) out[e] = src[f][g];
        else mout[(size_t)(f - nf) * nc + r] = msrc[f - nf][g];
    }
}

// Scatter an ice-grid field into the padded grid: background outside the crop.
__global__ void __launch_bounds__(NT)
k_out2in(double* __restrict__ dst, const double* __restrict__ src, Dom d, double background, int keep_outside)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < d.n; e += (size_t)gridDim.x * NT) {
        const int i = (int)(e % d.nx), j = (int)(e / d.nx);
        if (in_crop(d, i, j)) dst[e] = src[(size_t)(j - d.j0) * d.nxi + (i - d.i0)];
        else if (!keep_outside) dst[e] = background;
    }
}

// calc_z_ss, calc_Haf and calc_masks of one state (isos_init_state)
__global__ void __launch_bounds__(NT)
k_state_diag(double* z_ss, const double* zss_base, const double* dz_ss, double bsl, const double* z_bed,
             const double* Hice, double* Haf, uint8_t* mo, uint8_t* mg, uint8_t* mc, size_t n, double rho_sw_over_ice)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
        const double zss = (bsl + zss_base[e]) + dz_ss[e];
        z_ss[e] = zss;
        double h = (zss - z_bed[e]) * rho_sw_over_ice;
        if (h < 0.0) h = 0.0;
        h = Hice[e] - h;
        if (h < 0.0) h = 0.0;
        Haf[e] = h;
        const bool cont = z_bed[e] > zss;
        const bool grd = (Hice[e] > 0.0) && (h > 0.0);
        mc[e] = cont;
        mg[e] = grd;
        mo[e] = !(cont || grd);
    }
}

// ---------------------------------------------------------------------------
static int grid_for(size_t n)
{
    size_t b = (n + NT - 1) / NT;
    if (b > 152 * 8) b = 152 * 8;
    if (b < 1) b = 1;
    return (int)b;
}

// ---- LLRA / LV-ELRA (methods 0-2) ---------------------------------------
// Equilibrium displacement (src/lv_xlra.f90:30-39, src/fastisostasy.f90:
// 685-715) and relaxation rate (w_eq - w) / tau (src/lv_xlra.f90:17-27).
__global__ void __launch_bounds__(NT) k_weq_local(double* __restrict__ weq, const double* __restrict__ c_load,
                                                  double rho_m, int zero, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
        weq[e] = zero ? 0.0 : -c_load[e] / rho_m;
}

// the LV-ELRA load -canom_load g K^2 for the convolution with GV
template <typename T>
__global__ void __launch_bounds__(NT) k_elra_load(T* __restrict__ in, const double* __restrict__ c_load,
                                                  const double* __restrict__ K2, double g, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
        in[e] = (T)((-c_load[e] * g) * K2[e]);
}

// w_eq = (conv - mean of the padded buffer's corners), then the domain's own
// corner BC (apply_zerobc_at_corners on w_equilibrium)
__global__ void __launch_bounds__(NT) k_weq_elra(double* __restrict__ weq, const double* __restrict__ raw,
                                                 const double* __restrict__ corners, int nx, int ny)
{
    __shared__ double s_c[2];
    if (threadIdx.x == 0) {
        const double c1 = corner_mean(corners[0], corners[1], corners[2], corners[3]);
        const size_t last = (size_t)(ny - 1) * nx;
        s_c[0] = c1;
        s_c[1] = corner_mean(raw[0] - c1, raw[last + nx - 1] - c1, raw[last] - c1, raw[nx - 1] - c1);
    }
    __syncthreads();
    const double c1 = s_c[0], c2 = s_c[1];
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
        weq[e] = (raw[e] - c1) - c2;
}

template <typename T>
__global__ void __launch_bounds__(NT) k_relax_rate(T* __restrict__ out, const double* __restrict__ y,
                                                   const double* __restrict__ weq, double tau, size_t n,
                                                   const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
        out[e] = (T)((weq[e] - y[e]) / tau);
}

void weq_local(double* weq, const double* c_load, double rho_m, int zero, size_t n, cudaStream_t s)
{
    k_weq_local<<<grid_for(n), NT, 0, s>>>(weq, c_load, rho_m, zero, n);
}
template <typename T> void elra_load(T* in, const double* c_load, const double* K2, double g, size_t n, cudaStream_t s)
{
    k_elra_load<T><<<grid_for(n), NT, 0, s>>>(in, c_load, K2, g, n);
}
void weq_elra(double* weq, const double* raw, const double* corners, int nx, int ny, cudaStream_t s)
{
    k_weq_elra<<<grid_for((size_t)nx * ny), NT, 0, s>>>(weq, raw, corners, nx, ny);
}
template <typename T>
void relax_rate(T* out, const double* y, const double* weq, double tau, size_t n, const int* gate, cudaStream_t s)
{
    k_relax_rate<T><<<grid_for(n), NT, 0, s>>>(out, y, weq, tau, n, gate);
}
template void elra_load<float>(float*, const double*, const double*, double, size_t, cudaStream_t);
template void elra_load<double>(double*, const double*, const double*, double, size_t, cudaStream_t);
template void relax_rate<float>(float*, const double*, const double*, double, size_t, const int*, cudaStream_t);
template void relax_rate<double>(double*, const double*, const double*, double, size_t, const int*, cudaStream_t);

int reduce_grid(size_t n) { return grid_for(n); }

// Tsit5 attempt kernels: about 8 cells per thread, so that the per-thread
// partial sums and maxima of the mixed form stay in FP32 and only block
// totals pass through FP64.
int ts_grid(size_t n)
{
    size_t b = (n + (size_t)NT * 8 - 1) / ((size_t)NT * 8);
    if (b > 152 * 8) b = 152 * 8;
    if (b < 1) b = 1;
    return (int)b;
}

// ---- batched Tsit5 attempt over the members of an ensemble -----------------
template <typename T>
__global__ void __launch_bounds__(NT) k_b_ts_max(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { return M[m].d.ctl->done == 0; }, [&](int m, int local) {
        const BMember& b = M[m];
        ts_max_body<T>(b.d, (const T*)b.raw, b.atol, b.rtol, local, b.red_nblk);
        __syncthreads();
    });
}

template <typename T>
__global__ void __launch_bounds__(NT)
k_b_ts_err(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { return M[m].d.ctl->done == 0; }, [&](int m, int local) {
        const BMember& b = M[m];
        ts_err_body<T>(b.d, (const T*)b.raw, b.q, b.dt_max, local, b.red_nblk);
        __syncthreads();
    });
}

template <typename T>
__global__ void __launch_bounds__(NT) k_b_ts_commit(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { const Ctl* c = M[m].d.ctl; return c->done == 0 && c->accepted != 0; },
               [&](int m, int local) {
                   const BMember& b = M[m];
                   if (b.yhi) ts_commit_tpair_body(b.d, b.xhi, b.xlo, b.xdw, b.yhi, b.ylo, b.ydw, local, b.red_nblk);
                   else ts_commit_body<T>(b.d, (const T*)b.raw, local, b.red_nblk);
               });
}

__global__ void __launch_bounds__(NT)
k_b_ts_fused(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { return M[m].d.ctl->done == 0; }, [&](int m, int local) {
        const BMember& b = M[m];
        ts_fused_body(b.d, (const float*)b.raw, b.atol, b.rtol, b.q, b.dt_max, local, b.red_nblk);
        __syncthreads();
    });
}

__global__ void __launch_bounds__(NT) k_b_ts_commit_pair(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { const Ctl* c = M[m].d.ctl; return c->done == 0 && c->accepted != 0; },
               [&](int m, int local) {
                   const BMember& b = M[m];
                   ts_commit_pair_body(b.d, (const float*)b.raw, local, b.red_nblk);
               });
}

template <typename T> __device__ __forceinline__ DPRaw<T> member_raw(const BMember& b)
{
    DPRaw<T> r;
#pragma unroll
    for (int q = 0; q < 7; ++q) r.p[q] = (const T*)b.raw7[q];
    return r;
}

template <typename T>
__global__ void __launch_bounds__(NT) k_b_dp_stage(const BMember* __restrict__ M, BList L, int i)
{
    batch_walk(L, [&](int m) { return M[m].d.ctl->done == 0; }, [&](int m, int local) {
        const BMember& b = M[m];
        if constexpr (sizeof(T) == 4) {
            if (b.yhi) {   // mixed members: the stage state as a float pair
                dp_stage_pair_body(b.d.ctl, b.xhi, b.xlo, b.wrhi, b.wrlo, b.yhi, b.ylo, b.ydw,
                                   i == 6 ? b.d.ts_x2 : nullptr, b.d.x, member_raw<T>(b), i, b.p.nx, b.p.ny, b.d.spy,
                                   local, b.red_nblk);
                __syncthreads();
                return;
            }
        }
        dp_stage_body<T>(b.d.ctl, i == 6 ? b.d.ts_x2 : b.yst, b.d.x, member_raw<T>(b), i, b.p.nx, b.p.ny, b.d.spy,
                         local, b.red_nblk);
        __syncthreads();
    });
}

template <typename T>
__global__ void __launch_bounds__(NT) k_b_dp_err(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { return M[m].d.ctl->done == 0; }, [&](int m, int local) {
        const BMember& b = M[m];
        dp_err_body<T>(b.d, member_raw<T>(b), b.atol, b.rtol, local, b.red_nblk);
        __syncthreads();
    });
}

// accepted: the last stage's RHS becomes the next attempt's first (FSAL)
template <typename T>
__global__ void __launch_bounds__(NT) k_b_fsal(const BMember* __restrict__ M, BList L)
{
    batch_walk(L, [&](int m) { const Ctl* c = M[m].d.ctl; return c->done == 0 && c->accepted != 0; },
               [&](int m, int local) {
                   const BMember& b = M[m];
                   T* k0 = (T*)b.raw7[0];
                   const T* k6 = (const T*)b.raw7[6];
                   for (size_t e = (size_t)local * NT + threadIdx.x; e < b.d.n; e += (size_t)b.red_nblk * NT)
                       k0[e] = k6[e];
               });
}

template <typename T> void batch_dp_stage(const BMember* M, BList L, int nblk, int i, cudaStream_t s)
{
    k_b_dp_stage<T><<<nblk, NT, 0, s>>>(M, L, i);
}
template <typename T> void batch_dp_err(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_dp_err<T><<<nblk, NT, 0, s>>>(M, L);
}
template <typename T> void batch_fsal(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_fsal<T><<<nblk, NT, 0, s>>>(M, L);
}
template void batch_dp_stage<float>(const BMember*, BList, int, int, cudaStream_t);
template void batch_dp_stage<double>(const BMember*, BList, int, int, cudaStream_t);
template void batch_dp_err<float>(const BMember*, BList, int, cudaStream_t);
template void batch_dp_err<double>(const BMember*, BList, int, cudaStream_t);
template void batch_fsal<float>(const BMember*, BList, int, cudaStream_t);
template void batch_fsal<double>(const BMember*, BList, int, cudaStream_t);

template <typename T> int batch_red_resident()
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_ts_max<T>, NT, 0) != cudaSuccess || per < 1) per = 1;
    int p2 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p2, k_b_ts_err<T>, NT, 0) == cudaSuccess && p2 >= 1 && p2 < per)
        per = p2;
    if (sizeof(T) == 4 &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p2, k_b_ts_fused, NT, 0) == cudaSuccess && p2 >= 1 && p2 < per)
        per = p2;
    return per;
}
template int batch_red_resident<float>();
template int batch_red_resident<double>();

__global__ void k_b_loop_begin(const BMember* __restrict__ M, int nm)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nm) return;
    Ctl* c = M[m].d.ctl;
    c->rhs_valid = 0;
    c->have_rhs = 0;
    c->loop_iter = 0;
    c->need_rhs = 0;
}

// One block: attempt_begin of every member, then the compacted lists of the
// members that need an RHS (kinds 0-2) and that have an attempt (kind 3),
// with the prefix sums of their virtual blocks, in member order.
__global__ void k_b_attempt_begin(const BMember* __restrict__ M, int nm, int max_iter, const int* __restrict__ off,
                                  int* __restrict__ cl)
{
    extern __shared__ int sh_cl[];
    int* fl = sh_cl;        // bit 0: needs an RHS, bit 1: has an attempt
    int* cn = sh_cl + nm;   // virtual blocks of member m for kind k at cn[k nm + m]
    for (int m = threadIdx.x; m < nm; m += blockDim.x) {
        Ctl* c = M[m].d.ctl;
        attempt_begin_one(c, max_iter);
        fl[m] = (c->need_rhs ? 1 : 0) | (c->done == 0 ? 2 : 0);
#pragma unroll
        for (int k = 0; k < 4; ++k) cn[k * nm + m] = off[k * (nm + 1) + m + 1] - off[k * (nm + 1) + m];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int* idsR = cl + 2;
        int* idsT = cl + 2 + nm;
        int* co = cl + 2 + 2 * nm;
        int nR = 0, nT = 0, a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, a6 = 0;
        for (int k = 0; k < 7; ++k) co[k * (nm + 1)] = 0;
        for (int m = 0; m < nm; ++m) {
            const int f = fl[m];
            if (f & 1) {
                idsR[nR] = m;
                a0 += cn[m];
                a1 += cn[nm + m];
                a2 += cn[2 * nm + m];
                ++nR;
                co[nR] = a0;
                co[(nm + 1) + nR] = a1;
                co[2 * (nm + 1) + nR] = a2;
            }
            if (f & 2) {
                idsT[nT] = m;
                a3 += cn[3 * nm + m];
                a4 += cn[m];
                a5 += cn[nm + m];
                a6 += cn[2 * nm + m];
                ++nT;
                co[3 * (nm + 1) + nT] = a3;
                co[4 * (nm + 1) + nT] = a4;
                co[5 * (nm + 1) + nT] = a5;
                co[6 * (nm + 1) + nT] = a6;
            }
        }
        cl[0] = nR;
        cl[1] = nT;
    }
}

// continue while any member has an attempt left
__global__ void k_b_attempt_end(const BMember* __restrict__ M, int nm, cudaGraphConditionalHandle loop, int* more_out,
                                int fsal)
{
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    int more = 0;
    for (int m = threadIdx.x; m < nm; m += blockDim.x) more |= attempt_end_one(M[m].d.ctl, fsal);
    if (more) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (more_out) *more_out = any;
        else cudaGraphSetConditional(loop, any ? 1u : 0u);
    }
}

__global__ void k_b_set_args(const BArgs* __restrict__ a, int nm)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < nm) set_args_one(a[m].ctl, a[m].tf, a[m].bsl, a[m].A_ocean, a[m].method, a[m].write_bsl);
}

template <typename T> void batch_ts_max(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_ts_max<T><<<nblk, NT, 0, s>>>(M, L);
}
template <typename T>
void batch_ts_err(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_ts_err<T><<<nblk, NT, 0, s>>>(M, L);
}
void batch_ts_fused(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_ts_fused<<<nblk, NT, 0, s>>>(M, L);
}
void batch_ts_commit_pair(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_ts_commit_pair<<<nblk, NT, 0, s>>>(M, L);
}
template <typename T> void batch_ts_commit(const BMember* M, BList L, int nblk, cudaStream_t s)
{
    k_b_ts_commit<T><<<nblk, NT, 0, s>>>(M, L);
}
void batch_loop_begin(const BMember* M, int nm, cudaStream_t s) { k_b_loop_begin<<<(nm + 127) / 128, 128, 0, s>>>(M, nm); }
void batch_attempt_begin(const BMember* M, int nm, int max_iter, const int* off, int* cl, cudaStream_t s)
{
    k_b_attempt_begin<<<1, 256, 5 * (size_t)nm * sizeof(int), s>>>(M, nm, max_iter, off, cl);
}
void batch_attempt_end(const BMember* M, int nm, cudaGraphConditionalHandle loop, cudaStream_t s, int* more_out,
                       int fsal)
{
    k_b_attempt_end<<<1, 256, 0, s>>>(M, nm, loop, more_out, fsal);
}
void batch_set_args(const BArgs* a, int nm, cudaStream_t s) { k_b_set_args<<<(nm + 127) / 128, 128, 0, s>>>(a, nm); }
template void batch_ts_max<float>(const BMember*, BList, int, cudaStream_t);
template void batch_ts_max<double>(const BMember*, BList, int, cudaStream_t);
template void batch_ts_err<float>(const BMember*, BList, int, cudaStream_t);
template void batch_ts_err<double>(const BMember*, BList, int, cudaStream_t);
template void batch_ts_commit<float>(const BMember*, BList, int, cudaStream_t);
template void batch_ts_commit<double>(const BMember*, BList, int, cudaStream_t);

int reduce_blocks(size_t n) { return grid_for(n); }

// Kernels ending in a grid reduction: two blocks of NT per SM, each thread
// looping over several cells, so the per-thread shuffle tree of the block
// reduction is paid once per several cells (at most reduce_blocks blocks).
static int red_grid(size_t n)
{
    const int g = grid_for(n);
    return g < 152 * 2 ? g : 152 * 2;
}

void upd_begin(const Dom& d, const double* H_ice, cudaStream_t s)
{
    k_upd_begin<<<red_grid(d.n), NT, 0, s>>>(d, H_ice);
}
template <typename T> void upd_masks(const Dom& d, T* conv_in, cudaStream_t s)
{
    k_upd_masks<T><<<grid_for(d.n), NT, 0, s>>>(d, conv_in);
}
template <typename T>
void upd_litho(const Dom& d, const double* we_raw, const double* corners, int we_mode, T* conv_in, cudaStream_t s)
{
    k_upd_litho<T><<<grid_for(d.n), NT, 0, s>>>(d, we_raw, corners, we_mode, conv_in);
}
template <typename T>
void upd_load(const Dom& d, const double* dz_raw, const double* corners, int dz_mode, T* q0, int stage_mode,
              int run_integrator, cudaStream_t s)
{
    k_upd_load<T><<<grid_for(d.n), NT, 0, s>>>(d, dz_raw, corners, dz_mode, q0, stage_mode, run_integrator);
}
void set_args(Ctl* c, double tf, double bsl, double A_ocean, int method, int write_bsl, cudaStream_t s)
{
    k_set_args<<<1, 32, 0, s>>>(c, tf, bsl, A_ocean, method, write_bsl);
}
void step_begin(Ctl* c, int kind, cudaStream_t s) { k_step_begin<<<1, 32, 0, s>>>(c, kind); }
void step_end(Ctl* c, cudaStream_t s) { k_step_end<<<1, 32, 0, s>>>(c); }
void ts_loop_begin(Ctl* c, cudaStream_t s) { k_ts_loop_begin<<<1, 32, 0, s>>>(c); }
void ts_attempt_begin(Ctl* c, int max_iter, cudaStream_t s) { k_ts_attempt_begin<<<1, 32, 0, s>>>(c, max_iter); }
void ts_attempt_end(Ctl* c, cudaGraphConditionalHandle loop, cudaStream_t s, int fsal, int* more_out)
{
    k_ts_attempt_end<<<1, 32, 0, s>>>(c, loop, fsal, more_out);
}
template <typename T>
void dp_stage(const Ctl* c, double* y, const double* x, const DPRaw<T>& r, int i, int nx, int ny, double spy,
              cudaStream_t s)
{
    k_dp_stage<T><<<grid_for((size_t)nx * ny), NT, 0, s>>>(c, y, x, r, i, nx, ny, spy);
}
template <typename T> void dp_err(const Dom& d, const DPRaw<T>& r, double atol, double rtol, cudaStream_t s)
{
    k_dp_err<T><<<ts_grid(d.n), NT, 0, s>>>(d, r, atol, rtol);
}
template <typename T> void fsal_copy(const Ctl* c, T* k0, const T* k6, size_t n, cudaStream_t s)
{
    k_fsal_copy<T><<<grid_for(n), NT, 0, s>>>(c, k0, k6, n);
}
template void dp_stage<float>(const Ctl*, double*, const double*, const DPRaw<float>&, int, int, int, double,
                              cudaStream_t);
template void dp_stage<double>(const Ctl*, double*, const double*, const DPRaw<double>&, int, int, int, double,
                               cudaStream_t);
template void dp_err<float>(const Dom&, const DPRaw<float>&, double, double, cudaStream_t);
template void dp_err<double>(const Dom&, const DPRaw<double>&, double, double, cudaStream_t);
template void fsal_copy<float>(const Ctl*, float*, const float*, size_t, cudaStream_t);
template void fsal_copy<double>(const Ctl*, double*, const double*, size_t, cudaStream_t);
template <typename T>
void rk_stage(const Ctl* c, double* y, const double* x, const T* raw, double a, int nx, int ny, double spy,
              cudaStream_t s)
{
    k_rk_stage<T><<<grid_for((size_t)nx * ny), NT, 0, s>>>(c, y, x, raw, a, nx, ny, spy);
}
template <typename T>
void rk4_final(Ctl* c, double* x, double* w, const T* r1, const T* r2, const T* r3, const T* r4, int nx, int ny,
               double spy, cudaStream_t s)
{
    k_rk4_final<T><<<grid_for((size_t)nx * ny), NT, 0, s>>>(c, x, w, r1, r2, r3, r4, nx, ny, spy);
}
void dp_stage_pair(const Ctl* c, const float* xhi, const float* xlo, const float* wrhi, const float* wrlo, float* yhi,
                   float* ylo, float* ydw, double* x2, const double* x, const DPRaw<float>& r, int i, int nx, int ny,
                   double spy, cudaStream_t s)
{
    k_dp_stage_pair<<<grid_for((size_t)nx * ny), NT, 0, s>>>(c, xhi, xlo, wrhi, wrlo, yhi, ylo, ydw, x2, x, r, i, nx,
                                                             ny, spy);
}
void ts_commit_tpair(const Dom& d, float* xhi, float* xlo, float* xdw, const float* yhi, const float* ylo,
                     const float* ydw, cudaStream_t s)
{
    k_ts_commit_tpair<<<ts_grid(d.n), NT, 0, s>>>(d, xhi, xlo, xdw, yhi, ylo, ydw);
}
void rk4_final_pair(Ctl* c, double* x, double* w, float* xhi, float* xlo, const float* wrhi, const float* wrlo,
                    float* dxw, const float* r1, const float* r2, const float* r3, const float* r4, int nx, int ny,
                    double spy, cudaStream_t s)
{
    k_rk4_final_pair<<<grid_for((size_t)nx * ny), NT, 0, s>>>(c, x, w, xhi, xlo, wrhi, wrlo, dxw, r1, r2, r3, r4, nx,
                                                              ny, spy);
}
template <typename T>
void euler_final(const Ctl* c, double* x, double* w, const T* r1, int nx, int ny, double spy, cudaStream_t s)
{
    k_euler_final<T><<<grid_for((size_t)nx * ny), NT, 0, s>>>(c, x, w, r1, nx, ny, spy);
}
template <typename T> void ts_max(const Dom& d, const T* raw, double atol, double rtol, cudaStream_t s)
{
    k_ts_max<T><<<ts_grid(d.n), NT, 0, s>>>(d, raw, atol, rtol);
}
template <typename T> void ts_err(const Dom& d, const T* raw, double q, double dt_max, cudaStream_t s)
{
    k_ts_err<T><<<ts_grid(d.n), NT, 0, s>>>(d, raw, q, dt_max);
}
template <typename T> void ts_commit(const Dom& d, const T* raw, cudaStream_t s)
{
    k_ts_commit<T><<<ts_grid(d.n), NT, 0, s>>>(d, raw);
}
void ts_fused(const Dom& d, const float* raw, double atol, double rtol, double q, double dt_max,
              cudaStream_t s)
{
    k_ts_fused<<<ts_grid(d.n), NT, 0, s>>>(d, raw, atol, rtol, q, dt_max);
}
void ts_commit_pair(const Dom& d, const float* raw, cudaStream_t s)
{
    k_ts_commit_pair<<<ts_grid(d.n), NT, 0, s>>>(d, raw);
}
template <typename T> void upd_end(const Dom& d, const T* raw_last, int have_rhs, cudaStream_t s)
{
    k_upd_end<T><<<red_grid(d.n), NT, 0, s>>>(d, raw_last, have_rhs);
    k_copy<<<grid_for(d.n), NT, 0, s>>>(d.w, d.wout, d.n);
}
void gather(const double* const* src, const uint8_t* const* msrc, int nf, int nm, const Dom& d, double* out,
            cudaStream_t s)
{
    k_gather<<<grid_for((size_t)d.nxi * d.nyi * (nf + nm)), NT, 0, s>>>(src, msrc, nf, nm, d, out);
}
void gather_bytes(const double* const* src, const uint8_t* const* msrc, int nf, int nm, const Dom& d, double* out,
                  uint8_t* mout, cudaStream_t s)
{
    k_gather_bytes<<<grid_for((size_t)d.nxi * d.nyi * (nf + nm)), NT, 0, s>>>(src, msrc, nf, nm, d, out, mout);
}
void out2in(double* dst, const double* src, const Dom& d, double background, int keep_outside, cudaStream_t s)
{
    k_out2in<<<grid_for(d.n), NT, 0, s>>>(dst, src, d, background, keep_outside);
}
void state_diag(double* z_ss, const double* zss_base, const double* dz_ss, double bsl, const double* z_bed,
                const double* Hice, double* Haf, uint8_t* mo, uint8_t* mg, uint8_t* mc, size_t n,
                double rho_sw_over_ice, cudaStream_t s)
{
    k_state_diag<<<grid_for(n), NT, 0, s>>>(z_ss, zss_base, dz_ss, bsl, z_bed, Hice, Haf, mo, mg, mc, n,
                                             rho_sw_over_ice);
}


// --- small helpers for the single-function entry points ---------------------
template <typename T>
__global__ void __launch_bounds__(NT) k_rhs_finish(double* __restrict__ out, const T* __restrict__ raw, int nx, int ny,
                                                   double spy)
{
    const double cm = block_corner_mean(raw, nx, ny);
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
        out[e] = ((double)raw[e] - cm) * spy;
}

__global__ void __launch_bounds__(NT) k_sub_corner(double* __restrict__ out, const double* __restrict__ raw,
                                                   const double* __restrict__ corners, size_t n)
{
    const double cm = corner_mean(corners[0], corners[1], corners[2], corners[3]);
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) out[e] = raw[e] - cm;
}

template <typename T>
__global__ void __launch_bounds__(NT) k_cast(T* __restrict__ dst, const double* __restrict__ src, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) dst[e] = (T)src[e];
}

template <typename T>
__global__ void __launch_bounds__(NT) k_q0_from_cf(T* __restrict__ q0, const double* __restrict__ cf,
                                                   const uint8_t* __restrict__ mask, double g, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
        q0[e] = (T)(mask[e] ? -g * cf[e] : 0.0);
}

template <typename T> void rhs_finish(double* out, const T* raw, int nx, int ny, double spy, cudaStream_t s)
{
    k_rhs_finish<T><<<grid_for((size_t)nx * ny), NT, 0, s>>>(out, raw, nx, ny, spy);
}
void sub_corner(double* out, const double* raw, const double* corners, size_t n, cudaStream_t s)
{
    k_sub_corner<<<grid_for(n), NT, 0, s>>>(out, raw, corners, n);
}
template <typename T> void cast_from_double(T* dst, const double* src, size_t n, cudaStream_t s)
{
    k_cast<T><<<grid_for(n), NT, 0, s>>>(dst, src, n);
}
template <typename T> void q0_from_cf(T* q0, const double* cf, const uint8_t* mask, double g, size_t n, cudaStream_t s)
{
    k_q0_from_cf<T><<<grid_for(n), NT, 0, s>>>(q0, cf, mask, g, n);
}

#define FI_STATE_INST(T)                                                                                      \
    template void upd_masks<T>(const Dom&, T*, cudaStream_t);                                                 \
    template void upd_litho<T>(const Dom&, const double*, const double*, int, T*, cudaStream_t);              \
    template void upd_load<T>(const Dom&, const double*, const double*, int, T*, int, int, cudaStream_t);     \
    template void rk_stage<T>(const Ctl*, double*, const double*, const T*, double, int, int, double, cudaStream_t); \
    template void rk4_final<T>(Ctl*, double*, double*, const T*, const T*, const T*, const T*, int, int, double,  \
                               cudaStream_t);                                                                 \
    template void euler_final<T>(const Ctl*, double*, double*, const T*, int, int, double, cudaStream_t);     \
    template void ts_max<T>(const Dom&, const T*, double, double, cudaStream_t);                              \
    template void ts_err<T>(const Dom&, const T*, double, double, cudaStream_t);                              \
    template void ts_commit<T>(const Dom&, const T*, cudaStream_t);                                           \
    template void upd_end<T>(const Dom&, const T*, int, cudaStream_t);                                       \
    template void rhs_finish<T>(double*, const T*, int, int, double, cudaStream_t);                          \
    template void cast_from_double<T>(T*, const double*, size_t, cudaStream_t);                               \
    template void q0_from_cf<T>(T*, const double*, const uint8_t*, double, size_t, cudaStream_t);

FI_STATE_INST(double)
FI_STATE_INST(float)

}  // namespace fi
