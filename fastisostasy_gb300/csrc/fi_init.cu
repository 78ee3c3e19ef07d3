// fi_init.cu — init-time fields computed on the device.
//
// calc_kappa (src/lv_elva.f90:442-481), the elastic Green's function
// (calc_elastic_green with get_ge_value, src/green_functions.f90:43-91,
// 131-168) and the geoid Green's function (calc_z_ss_green with
// calc_gn_value, :94-128, 171-181) are the cell-by-cell part of isos_init
// that grows with the domain: one thread per cell here instead of a host
// loop, the results copied back for the host-side set-up that follows.
#include <cmath>
#include <vector>

#include <cuda_runtime.h>

#include "fi_init.h"

namespace fi {

__constant__ float c_ge_rn[42];
__constant__ float c_ge_v[42];

__device__ double ge_value_dev(double r)
{
    // the table's radii are scaled by 1.e3 in single precision
    const double rlast = (double)(c_ge_rn[41] * 1.e3f);
    if (r > rlast) return 0.0;
    int k = 0;
    while (k < 41 && !(r >= (double)(c_ge_rn[k] * 1.e3f) && r < (double)(c_ge_rn[k + 1] * 1.e3f))) ++k;
    if (k > 40) k = 40;
    const double r0 = (double)(c_ge_rn[k] * 1.e3f), r1 = (double)(c_ge_rn[k + 1] * 1.e3f);
    const double g0 = (double)c_ge_v[k], g1 = (double)c_ge_v[k + 1];
    // unfused, in the order written: the same bits as the host evaluation
    return __dadd_rn(g0, __dmul_rn(__ddiv_rn(__dsub_rn(r, r0), __dsub_rn(r1, r0)), __dsub_rn(g1, g0)));
}

__global__ void k_init_fields(double* __restrict__ kappa, double* __restrict__ GE, double* __restrict__ GN, int nx,
                              int ny, double dx, double mu_x, double mu_y, double ge_scale, double g_lit,
                              double r_earth, double m_earth)
{
    const int ic = (nx - 1) / 2 + 1, jc = (ny - 1) / 2 + 1;
    const int mx = (nx % 2 == 0) ? nx / 2 : (nx - 1) / 2;   // midindex, used for x and y alike
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % nx) + 1, j = (int)(e / nx) + 1;
        const double pp = (i <= ic) ? mu_x * (i - 1) : mu_x * (nx - i + 1);
        const double q = (j <= jc) ? mu_y * (j - 1) : mu_y * (ny - j + 1);
        // products and sums unfused (no FMA contraction), as on the host
        kappa[e] = sqrt(__dadd_rn(__dmul_rn(pp, pp), __dmul_rn(q, q)));   // x**0.5, correctly rounded
        const double x = (i - 1 - mx) * dx, y = (j - 1 - mx) * dx;
        const double r = sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
        GE[e] = __dmul_rn(__dmul_rn(ge_value_dev(r), ge_scale), __dmul_rn(dx, dx)) / __dmul_rn(g_lit, (r > dx ? r : dx));
        const double rr = (dx / 2 > r) ? dx / 2 : r;
        // the device sine may differ from the C library's in the last place
        GN[e] = r_earth / __dmul_rn(__dmul_rn(2., m_earth), sin(rr / (2. * r_earth)));
    }
}

int init_fields_device(int nx, int ny, double dx, double dy, double pi_lit, double ge_scale, double g_lit,
                       double r_earth, double m_earth, const float* ge_rn, const float* ge_v, double* kappa,
                       double* GE, double* GN, cudaStream_t s)
{
    const size_t n = (size_t)nx * ny;
    double* buf = nullptr;
    // stream-ordered: set-up of one handle never waits for other handles' work
    if (cudaMallocAsync((void**)&buf, 3 * n * sizeof(double), s) != cudaSuccess) return 1;
    int rc = 0;
    if (cudaMemcpyToSymbolAsync(c_ge_rn, ge_rn, 42 * sizeof(float), 0, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyToSymbolAsync(c_ge_v, ge_v, 42 * sizeof(float), 0, cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = 1;
    if (!rc) {
        const double mu_x = 2.0 * pi_lit / ((nx - 1) * dx), mu_y = 2.0 * pi_lit / ((ny - 1) * dy);
        int blocks = (int)((n + 255) / 256);
        if (blocks > 152 * 16) blocks = 152 * 16;
        k_init_fields<<<blocks, 256, 0, s>>>(buf, buf + n, buf + 2 * n, nx, ny, dx, mu_x, mu_y, ge_scale, g_lit,
                                             r_earth, m_earth);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(kappa, buf, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(GE, buf + n, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(GN, buf + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = 1;
    }
    cudaFreeAsync(buf, s);
    if (!rc) kappa[0] = (kappa[nx] + kappa[1]) / 2.0;   // kappa(1,1), src/lv_elva.f90:478
    return rc;
}

// ---- rheology --------------------------------------------------------------

constexpr int kGrid = 152 * 8;

__device__ __forceinline__ void cell_ij(size_t e, int nx, int& i, int& j)
{
    i = (int)(e % nx);
    j = (int)(e / nx);
}

// calc_gaussian_thickness / calc_gaussian_viscosity core
// (src/isos_utils.f90:960-1035): exp(-1/2 d^T S d), S = diag((4/Lx)^2, (4/Ly)^2)
__global__ void k_gauss(double* __restrict__ g, const double* __restrict__ xc, const double* __restrict__ yc, int nx,
                        int ny, double xcntr, double ycntr, double s11, double s22)
{
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        int i, j;
        cell_ij(e, nx, i, j);
        const double d1 = xc[i] - xcntr, d2 = yc[j] - ycntr;
        g[e] = exp(-0.5 * (d1 * (s11 * d1 + 0.0 * d2) + d2 * (0.0 * d1 + s22 * d2)));
    }
}

// max (is_min = 0) or min (1) of positive doubles: their bit patterns order
// like the values
__global__ void k_extreme_pos(const double* __restrict__ a, size_t n, int is_min, unsigned long long* out)
{
    unsigned long long v = is_min ? ~0ull : 0ull;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(a[e]);
        v = is_min ? (b < v ? b : v) : (b > v ? b : v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = is_min ? (w < v ? w : v) : (w > v ? w : v);
    }
    if ((threadIdx.x & 31) == 0) {
        if (is_min) atomicMin(out, v);
        else atomicMax(out, v);
    }
}

// he_mode 0: He as it is (from the file), 1: uniform he0, 2: he0 + amp g / max g
__global__ void k_he_rigidity(double* __restrict__ He, double* __restrict__ D, const double* __restrict__ g,
                              const unsigned long long* __restrict__ gmax, size_t n, int he_mode, double he0,
                              double amp, double E, double nu)
{
    const double mx = he_mode == 2 ? __longlong_as_double((long long)*gmax) : 1.0;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        if (he_mode == 2) He[e] = he0 + amp * (g[e] / mx);
        else if (he_mode == 1) He[e] = he0;
        const double h = He[e];
        // calc_heterogeneous_rigidity (src/isos_utils.f90:90-100)
        D[e] = E * 1e9 * (h * h * h) / (12.0 * (1.0 - nu * nu));
    }
}

struct LumpArgs {
    int nl, layering, lumping;
    double zl[8], visc[8], dl;
};

// layer boundaries (calc_parallel / calc_equalized_layerboundaries,
// src/lv_elva.f90:131-168) and calc_effective_viscosity with
// calc_viscosity_scaling_freqdomain (src/lv_elva.f90:207-306); eta3 null:
// the layer viscosities of the parameter vector in every cell.
__global__ void k_lump(double* __restrict__ eta_eff, double* __restrict__ R, const double* __restrict__ He,
                       const double* __restrict__ kappa, const double* __restrict__ eta3, size_t n, LumpArgs a)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        double bnd[8], eta[8];
        bnd[0] = He[e];
        for (int k = 1; k < a.nl; ++k) bnd[k] = (a.layering == 1) ? bnd[k - 1] + a.dl : a.zl[k];
        for (int k = 0; k < a.nl; ++k) eta[k] = eta3 ? eta3[(size_t)k * n + e] : a.visc[k];
        double mn = eta[0], mxv = eta[0], sm = 0.0, ls = 0.0;
        for (int k = 0; k < a.nl; ++k) {
            mn = eta[k] < mn ? eta[k] : mn;
            mxv = eta[k] > mxv ? eta[k] : mxv;
            sm += eta[k];
            ls += log10(eta[k]);
        }
        double v = eta[a.nl - 1];
        switch (a.lumping) {
        case 1: v = mn; break;
        case 2: v = mxv; break;
        case 3: v = sm / (double)a.nl; break;
        case 4: v = pow(10.0, ls / (double)a.nl); break;
        default: break;
        }
        double r = 1.0;
        if (a.lumping == 5 && a.nl > 1) {
            for (int k = a.nl - 1; k >= 1; --k) {
                const double dz = bnd[k] - bnd[k - 1];
                const double er = eta[k - 1] / v, ir = 1. / er;
                const double kz = dz * kappa[e];
                const double c = cosh(kz), sn = sinh(kz);
                r = r * (2 * er * c * sn + (1 - er * er) * (kz * kz) + (er * sn) * (er * sn) + c * c) /
                    ((er + ir) * c * sn + (er - ir) * dz * kappa[e] + sn * sn + c * c);
            }
        }
        eta_eff[e] = v;
        R[e] = r;
    }
}

__global__ void k_eta_gauss(double* __restrict__ eta_eff, double* __restrict__ R, const double* __restrict__ g,
                            size_t n, double eta0, double sgn)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        eta_eff[e] = eta0 * pow(10.0, sgn * g[e]);
        R[e] = 1.0;
    }
}

// viscosity scaling (min / max / scale), compressibility, then
// exp(log10(eta_ref / eta)) * eta (src/fastisostasy.f90:425-442)
__global__ void k_eta_post(double* __restrict__ eta_eff, size_t n, int mode, const unsigned long long* __restrict__ ext,
                           double scale, double cc, double eta_ref)
{
    const double u = (mode == 2 || mode == 3) ? __longlong_as_double((long long)*ext) : 0.0;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        double v = eta_eff[e];
        if (mode == 2 || mode == 3) v = u;
        else if (mode == 1) v = v * scale;
        v = v * cc;
        eta_eff[e] = exp(log10(eta_ref / v)) * v;
    }
}

// bilinear_interpolation (src/isos_utils.f90:495-559) at every cell of the
// padded grid, in single precision as the routine declares its arguments
// (`real`); flat extension within 1 (unit of the coordinates) of the edges.
__global__ void k_bilinear(double* __restrict__ out, const float* __restrict__ z, const float* __restrict__ xr,
                           const float* __restrict__ yr, int nxr, int nyr, const double* __restrict__ xc,
                           const double* __restrict__ yc, int nx, int ny)
{
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        int ci, cj;
        cell_ij(e, nx, ci, cj);
        const float xo = (float)xc[ci], yo = (float)yc[cj], tol = 1.0f;
        bool flat = false;
        int i, j;
        float tx = 0.f, ty = 0.f;
        if (xo <= __fadd_rn(xr[0], tol)) { i = 0; flat = true; }
        else if (xo >= __fsub_rn(xr[nxr - 1], tol)) { i = nxr - 1; flat = true; }
        else {
            // first i with xr[i] < xo <= xr[i+1] (xr ascending)
            int lo = 0, hi = nxr - 2;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (xo <= xr[mid + 1]) hi = mid;
                else lo = mid + 1;
            }
            i = lo;
            tx = __fdiv_rn(__fsub_rn(xo, xr[i]), __fsub_rn(xr[i + 1], xr[i]));
        }
        if (yo <= __fadd_rn(yr[0], tol)) { j = 0; flat = true; }
        else if (yo >= __fsub_rn(yr[nyr - 1], tol)) { j = nyr - 1; flat = true; }
        else {
            int lo = 0, hi = nyr - 2;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (yo <= yr[mid + 1]) hi = mid;
                else lo = mid + 1;
            }
            j = lo;
            ty = __fdiv_rn(__fsub_rn(yo, yr[j]), __fsub_rn(yr[j + 1], yr[j]));
        }
        float zo;
        if (flat) {
            zo = z[(size_t)j * nxr + i];
        } else {
            const float z11 = z[(size_t)j * nxr + i], z21 = z[(size_t)j * nxr + i + 1];
            const float z12 = z[(size_t)(j + 1) * nxr + i], z22 = z[(size_t)(j + 1) * nxr + i + 1];
            const float ux = __fsub_rn(1.0f, tx), uy = __fsub_rn(1.0f, ty);
            float a = __fmul_rn(__fmul_rn(z11, ux), uy);
            a = __fadd_rn(a, __fmul_rn(__fmul_rn(z21, tx), uy));
            a = __fadd_rn(a, __fmul_rn(__fmul_rn(z12, ux), ty));
            a = __fadd_rn(a, __fmul_rn(__fmul_rn(z22, tx), ty));
            zo = a;
        }
        out[e] = (double)zo;
    }
}

// eta of layer l at every cell: interp_0d (src/isos_utils.f90:423-457) of
// the clamped log10 profile against depth, at the layer's boundary, then
// 10**(.) (src/fastisostasy.f90:362-406)
__global__ void k_vertical(double* __restrict__ eta3, const double* __restrict__ prof, const double* __restrict__ depth,
                           int nz, const double* __restrict__ He, size_t n, LumpArgs a)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        double b = He[e];
        for (int l = 0; l < a.nl; ++l) {
            if (l > 0) b = (a.layering == 1) ? b + a.dl : a.zl[l];
            double y;
            if (b < depth[0]) {
                y = prof[e];
            } else if (b > depth[nz - 1]) {
                y = prof[(size_t)(nz - 1) * n + e];
            } else {
                int jj = 0;
                while (jj < nz && !(depth[jj] >= b)) ++jj;
                if (jj == 0) y = prof[e];
                else if (jj == nz) y = prof[(size_t)(nz - 1) * n + e];
                else {
                    const double y0 = prof[(size_t)(jj - 1) * n + e], y1 = prof[(size_t)jj * n + e];
                    const double alpha = (b - depth[jj - 1]) / (depth[jj] - depth[jj - 1]);
                    y = y0 + alpha * (y1 - y0);
                }
            }
            eta3[(size_t)l * n + e] = pow(10.0, y);
        }
    }
}

// eta_bilin(.,.,k) += viscosity_scaling * stddev_bilin(.,.,k), then the
// clamp to [16, 23] (src/fastisostasy.f90:369-385)
__global__ void k_prof_clamp(double* __restrict__ prof, const double* __restrict__ sd, size_t m, double scale)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (size_t)gridDim.x * blockDim.x) {
        double v = prof[e];
        if (sd) v = v + scale * sd[e];
        if (v < 16) v = 16;
        if (v > 23) v = 23;
        prof[e] = v;
    }
}

// smooth_gauss_2D (src/isos_utils.f90:696-819) as two separable passes: the
// reference's normalised 2-D Gaussian window is the outer product of the
// normalised 1-D one (up to rounding), with the mirror extension
// (index 0 -> 1, nx+1 -> nx, 1-based) applied per axis.
__global__ void k_smooth_pass(double* __restrict__ out, const double* __restrict__ in, const double* __restrict__ w,
                              int n2, int nx, int ny, int along_y)
{
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        int i, j;
        cell_ij(e, nx, i, j);
        double acc = 0.0;
        for (int t = -n2; t <= n2; ++t) {
            int q = (along_y ? j : i) + t;
            const int m = along_y ? ny : nx;
            q = q < 0 ? -1 - q : (q >= m ? 2 * m - 1 - q : q);
            acc += w[t + n2] * (along_y ? in[(size_t)q * nx + i] : in[(size_t)j * nx + q]);
        }
        out[e] = acc;
    }
}

namespace {

// Scratch of one set-up call, stream-ordered (cudaMallocAsync /
// cudaFreeAsync on the handle's stream): no device-wide synchronisation, so
// handles created while others run (serving) do not stall them.
struct DevBuf {
    cudaStream_t s;
    std::vector<void*> p;
    explicit DevBuf(cudaStream_t st) : s(st) {}
    ~DevBuf()
    {
        for (void* q : p) cudaFreeAsync(q, s);
    }
    template <typename T> T* get(size_t count)
    {
        void* q = nullptr;
        if (cudaMallocAsync(&q, count * sizeof(T) + 16, s) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (T*)q;
    }
};

int grid_of(size_t n)
{
    size_t b = (n + 255) / 256;
    if (b > (size_t)kGrid) b = kGrid;
    return (int)(b < 1 ? 1 : b);
}

// normalised 1-D Gaussian weights of smooth_gauss_2D's window
void smooth_weights(double dx, double sigma, int n2, std::vector<double>& w)
{
    w.assign(2 * n2 + 1, 0.0);
    double sum = 0.0;
    for (int t = -n2; t <= n2; ++t) {
        const double x = t * dx;
        w[t + n2] = std::exp(-(x * x) / (2 * sigma * sigma));
        sum += w[t + n2];
    }
    for (double& v : w) v /= sum;
}

int smooth_device(double* f, double* tmp, int nx, int ny, double dx, double sigma, DevBuf& B, cudaStream_t s)
{
    const int n2 = (int)std::ceil(2.0 * sigma / dx);
    if (n2 >= nx || n2 >= ny) return 2;   // the mirror extension would leave points missing
    std::vector<double> w;
    smooth_weights(dx, sigma, n2, w);
    double* dw = B.get<double>(w.size());
    if (!dw || cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return 1;
    const size_t n = (size_t)nx * ny;
    k_smooth_pass<<<grid_of(n), 256, 0, s>>>(tmp, f, dw, n2, nx, ny, 0);
    k_smooth_pass<<<grid_of(n), 256, 0, s>>>(f, tmp, dw, n2, nx, ny, 1);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

int rheology_device(const RheoParams& P, const double* xc, const double* yc, double dx, const double* kappa,
                    const RheoFile* F, double* He_out, double* D_out, double* eta_out, double* R_out, cudaStream_t s)
{
    const int nx = P.nx, ny = P.ny;
    const size_t n = (size_t)nx * ny;
    const int G = grid_of(n);
    DevBuf B(s);
    double *dxc = B.get<double>(nx), *dyc = B.get<double>(ny), *He = B.get<double>(n), *D = B.get<double>(n);
    double *eta = B.get<double>(n), *R = B.get<double>(n), *tmp = B.get<double>(n);
    unsigned long long* ext = B.get<unsigned long long>(1);
    if (!dxc || !dyc || !He || !D || !eta || !R || !tmp || !ext) return 1;
    auto ck = [](cudaError_t e) { return e == cudaSuccess; };
    if (!ck(cudaMemcpyAsync(dxc, xc, nx * sizeof(double), cudaMemcpyHostToDevice, s)) ||
        !ck(cudaMemcpyAsync(dyc, yc, ny * sizeof(double), cudaMemcpyHostToDevice, s)))
        return 1;
    const double xcntr = (xc[nx - 1] + xc[0]) / 2.0, ycntr = (yc[ny - 1] + yc[0]) / 2.0;
    const double Lx = (xc[nx - 1] - xc[0]) / 2., Ly = (yc[ny - 1] - yc[0]) / 2.;
    const double s11 = (4.0 / Lx) * (4.0 / Lx), s22 = (4.0 / Ly) * (4.0 / Ly);
    // file grids in single precision, as bilinear_interpolation reads them
    auto upload_f = [&](const double* src, size_t cnt) -> float* {
        std::vector<float> h(cnt);
        for (size_t q = 0; q < cnt; ++q) h[q] = (float)src[q];
        float* d = B.get<float>(cnt);
        if (!d || !ck(cudaMemcpyAsync(d, h.data(), cnt * sizeof(float), cudaMemcpyHostToDevice, s)) ||
            !ck(cudaStreamSynchronize(s)))
            return nullptr;
        return d;
    };
    float *fxr = nullptr, *fyr = nullptr;
    if (F && (F->thick || F->log10_eta)) {
        if (F->nxr < 2 || F->nyr < 2 || !F->xr || !F->yr) return 2;
        if (!(fxr = upload_f(F->xr, F->nxr)) || !(fyr = upload_f(F->yr, F->nyr))) return 1;
    }
    // ---- lithosphere
    const double* gptr = nullptr;
    double he0 = P.zl[0], amp = 0.0;
    int he_mode = 1;
    if (F && F->thick) {
        std::vector<double> t((size_t)F->nxr * F->nyr);
        for (size_t q = 0; q < t.size(); ++q) t[q] = F->thick[q] * F->thick_scale;
        float* fz = upload_f(t.data(), t.size());
        if (!fz) return 1;
        k_bilinear<<<G, 256, 0, s>>>(He, fz, fxr, fyr, F->nxr, F->nyr, dxc, dyc, nx, ny);
        if (F->smooth_radius > 0.0) {
            const int rc = smooth_device(He, tmp, nx, ny, dx, F->smooth_radius, B, s);
            if (rc) return rc;
        }
        he_mode = 0;
    } else if (P.method == 3 && (P.lithosphere == 1 || P.lithosphere == 2)) {
        k_gauss<<<G, 256, 0, s>>>(tmp, dxc, dyc, nx, ny, xcntr, ycntr, s11, s22);
        const unsigned long long zero = 0ull;
        if (!ck(cudaMemcpyAsync(ext, &zero, sizeof(zero), cudaMemcpyHostToDevice, s))) return 1;
        k_extreme_pos<<<G, 256, 0, s>>>(tmp, n, 0, ext);
        gptr = tmp;
        amp = (P.lithosphere == 1 ? 1.0 : -1.0) * P.big_he;
        he_mode = 2;
    }
    k_he_rigidity<<<G, 256, 0, s>>>(He, D, gptr, ext, n, he_mode, he0, amp, P.E, P.nu);
    if (!ck(cudaGetLastError())) return 1;
    // ---- mantle
    LumpArgs la;
    la.nl = P.nl;
    la.layering = P.layering;
    la.lumping = P.lumping;
    la.dl = P.dl;
    for (int k = 0; k < 8; ++k) { la.zl[k] = P.zl[k]; la.visc[k] = P.viscosities[k]; }
    if (P.method == 3) {
        double* dk = B.get<double>(n);
        if (!dk || !ck(cudaMemcpyAsync(dk, kappa, n * sizeof(double), cudaMemcpyHostToDevice, s))) return 1;
        if (F && F->log10_eta) {
            const int nz = F->nzr;
            if (nz < 1 || !F->zr) return 2;
            // depth_rheo(i) = zc(nz) - zc(nz-i+1); level i of the profile is file level nz-i+1
            std::vector<double> depth(nz);
            for (int q = 0; q < nz; ++q) depth[q] = F->zr[nz - 1] - F->zr[nz - 1 - q];
            double* ddep = B.get<double>(nz);
            double* prof = B.get<double>((size_t)nz * n);
            double* sdp = (F->use_stddev && F->stddev) ? B.get<double>((size_t)nz * n) : nullptr;
            double* eta3 = B.get<double>((size_t)P.nl * n);
            if (!ddep || !prof || !eta3 || (F->use_stddev && F->stddev && !sdp) ||
                !ck(cudaMemcpyAsync(ddep, depth.data(), nz * sizeof(double), cudaMemcpyHostToDevice, s)))
                return 1;
            const size_t lev = (size_t)F->nxr * F->nyr;
            for (int q = 0; q < nz; ++q) {
                float* fz = upload_f(F->log10_eta + (size_t)(nz - 1 - q) * lev, lev);
                if (!fz) return 1;
                k_bilinear<<<G, 256, 0, s>>>(prof + (size_t)q * n, fz, fxr, fyr, F->nxr, F->nyr, dxc, dyc, nx, ny);
                if (sdp) {
                    float* fs = upload_f(F->stddev + (size_t)(nz - 1 - q) * lev, lev);
                    if (!fs) return 1;
                    k_bilinear<<<G, 256, 0, s>>>(sdp + (size_t)q * n, fs, fxr, fyr, F->nxr, F->nyr, dxc, dyc, nx, ny);
                }
            }
            k_prof_clamp<<<G, 256, 0, s>>>(prof, sdp, (size_t)nz * n, P.viscosity_scaling);
            k_vertical<<<G, 256, 0, s>>>(eta3, prof, ddep, nz, He, n, la);
            k_lump<<<G, 256, 0, s>>>(eta, R, He, dk, eta3, n, la);
            if (F->smooth_radius > 0.0) {
                const int rc = smooth_device(eta, tmp, nx, ny, dx, F->smooth_radius, B, s);
                if (rc) return rc;
            }
        } else if (P.mantle == 1 || P.mantle == 2) {
            // gaussian_plus passes yc = xc (src/fastisostasy.f90:329-330),
            // which covers the rows only on a square (or wider) grid
            if (P.mantle == 1 && ny > nx) return 2;
            k_gauss<<<G, 256, 0, s>>>(tmp, dxc, P.mantle == 1 ? dxc : dyc, nx, ny, xcntr, P.mantle == 1 ? xcntr : ycntr,
                                       s11, P.mantle == 1 ? s11 : s22);
            k_eta_gauss<<<G, 256, 0, s>>>(eta, R, tmp, n, P.viscosities[0], P.mantle == 1 ? 1.0 : -1.0);
        } else {
            // mantle 0: the parameter vector lumped; 3 (fields given later by
            // the caller): the bottom layer's value and R = 1 until then
            if (P.mantle == 3) la.lumping = 0;
            k_lump<<<G, 256, 0, s>>>(eta, R, He, dk, nullptr, n, la);
        }
        const int mode = (F && F->log10_eta && F->use_stddev) ? 0 : P.visc_scaling_method;
        if (mode == 2 || mode == 3) {
            const unsigned long long init = mode == 2 ? ~0ull : 0ull;
            if (!ck(cudaMemcpyAsync(ext, &init, sizeof(init), cudaMemcpyHostToDevice, s))) return 1;
            k_extreme_pos<<<G, 256, 0, s>>>(eta, n, mode == 2 ? 1 : 0, ext);
        }
        k_eta_post<<<G, 256, 0, s>>>(eta, n, mode, ext, P.viscosity_scaling, P.cc, P.eta_ref);
        if (!ck(cudaGetLastError())) return 1;
    }
    bool ok = true;
    if (He_out) ok = ok && ck(cudaMemcpyAsync(He_out, He, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (D_out) ok = ok && ck(cudaMemcpyAsync(D_out, D, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (P.method == 3) {
        if (eta_out) ok = ok && ck(cudaMemcpyAsync(eta_out, eta, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (R_out) ok = ok && ck(cudaMemcpyAsync(R_out, R, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    ok = ok && ck(cudaStreamSynchronize(s));
    return ok ? 0 : 1;
}

__global__ void k_narrow(const double2* __restrict__ a, float2* __restrict__ b, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const double2 v = a[e];
        b[e] = make_float2((float)v.x, (float)v.y);
    }
}

int narrow_spectrum(const double2* a, float2* b, size_t n, cudaStream_t s)
{
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_narrow<<<blocks, 256, 0, s>>>(a, b, n);
    return cudaGetLastError() != cudaSuccess;
}

}  // namespace fi
