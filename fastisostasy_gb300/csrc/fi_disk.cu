// fi_disk.cu — the analytical ELVA disc on the device, an in-run validator.
//
// Bueler et al. (2007), eq. 17, as the reference evaluates it for its disc
// benchmark (isosbench_elva_disk, src/isostasy_benchmarks.f90:74-127, and
// calc_analytical_viscous_disk, :131-280):
//
//   u(r, t) = int_0^0.1 rho_i g h0 r0 (exp(-beta t / (2 eta k)) - 1)
//                       J1(k r0) J0(k r) / beta  dk,   beta = rho_m g + D k^4
//
// with t in seconds (365 * 24 * 3600 per year).  The integral is a composite
// 8-point Gauss-Legendre rule on panels of 2e-7 over [0, 1e-3], where
// J1(k r0) oscillates, and 1e-4 over [1e-3, 0.1]; one block sums one radius
// (fixed order: deterministic).  The radial profile, sampled every dx, is
// put on the grid by the lower radius of each cell centre's distance and
// shifted by the mean of the four corners.
#include <cmath>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fi_gpu.h"

namespace {

constexpr int kGL = 8;

// Gauss-Legendre nodes and weights on [-1, 1] by Newton's method on P_n
void gauss_legendre(int n, double* x, double* w)
{
    for (int i = 0; i < n; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[n - 1 - i] = z;   // ascending
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

struct DiskArgs {
    double r0, h0, eta, D, rho_ice, rho_m, g, t_sec, dx;
    int npanel;
};

// profile[l] = u(l dx, t); block l, panels strided over the threads
__global__ void k_disk_profile(double* __restrict__ prof, const double* __restrict__ edges,
                               const double* __restrict__ gx, const double* __restrict__ gw, DiskArgs a)
{
    const double r = blockIdx.x * a.dx;
    double s = 0.0;
    for (int q = threadIdx.x; q < a.npanel; q += blockDim.x) {
        const double lo = edges[q], hi = edges[q + 1];
        const double half = 0.5 * (hi - lo), mid = 0.5 * (hi + lo);
        double ps = 0.0;
        for (int i = 0; i < kGL; ++i) {
            const double k = half * gx[i] + mid;
            const double beta = a.rho_m * a.g + a.D * (k * k) * (k * k);
            const double base = a.rho_ice * a.g * a.h0 * a.r0 * (exp(-beta * a.t_sec / (2.0 * a.eta * k)) - 1.0) *
                                j1(k * a.r0) / beta;
            ps += half * gw[i] * base * j0(k * r);
        }
        s += ps;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < (unsigned)st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) prof[blockIdx.x] = sh[0];
}

__global__ void k_disk_grid(double* __restrict__ out, const double* __restrict__ prof, int nx, int ny, double dx)
{
    const int ic = (nx - 1) / 2 + 1, jc = (ny - 1) / 2 + 1;
    const size_t n = (size_t)nx * ny;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % nx) + 1, j = (int)(e / nx) + 1;
        const double xi = dx * (i - ic), yj = dx * (j - jc);
        out[e] = prof[(int)std::floor(std::sqrt(xi * xi + yj * yj) / dx)];
    }
}

}  // namespace

extern "C" int fi_elva_disk(int nx, int ny, double dx, double r0, double h0, double eta, double D, double rho_ice,
                            double rho_m, double g, double time_yr, double* out)
{
    if (nx < 2 || ny < 2 || !(dx > 0.0) || !out) return FI_E_ARG;
    // panels: 5000 of 2e-7 on [0, 1e-3], 990 of 1e-4 on [1e-3, 0.1]
    std::vector<double> edges;
    for (int i = 0; i <= 5000; ++i) edges.push_back(1e-3 * i / 5000.0);
    for (int i = 1; i <= 990; ++i) edges.push_back(1e-3 + (0.1 - 1e-3) * i / 990.0);
    double gx[kGL], gw[kGL];
    gauss_legendre(kGL, gx, gw);
    const int nl = (int)((nx > ny ? nx : ny) * std::sqrt(2.0) / 2) + 2;
    const size_t n = (size_t)nx * ny;
    double *d_edges = nullptr, *d_gx = nullptr, *d_gw = nullptr, *d_prof = nullptr, *d_out = nullptr;
    int rc = FI_OK;
    if (cudaMalloc(&d_edges, edges.size() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&d_gx, sizeof(gx)) != cudaSuccess || cudaMalloc(&d_gw, sizeof(gw)) != cudaSuccess ||
        cudaMalloc(&d_prof, nl * sizeof(double)) != cudaSuccess || cudaMalloc(&d_out, n * sizeof(double)) != cudaSuccess)
        rc = FI_E_OOM;
    if (!rc && (cudaMemcpy(d_edges, edges.data(), edges.size() * sizeof(double), cudaMemcpyHostToDevice) ||
                cudaMemcpy(d_gx, gx, sizeof(gx), cudaMemcpyHostToDevice) ||
                cudaMemcpy(d_gw, gw, sizeof(gw), cudaMemcpyHostToDevice)))
        rc = FI_E_CUDA;
    if (!rc) {
        DiskArgs a;
        a.r0 = r0; a.h0 = h0; a.eta = eta; a.D = D; a.rho_ice = rho_ice; a.rho_m = rho_m; a.g = g;
        a.t_sec = time_yr * 365.0 * 24.0 * 3600.0;
        a.dx = dx;
        a.npanel = (int)edges.size() - 1;
        k_disk_profile<<<nl, 256>>>(d_prof, d_edges, d_gx, d_gw, a);
        k_disk_grid<<<(int)((n + 255) / 256), 256>>>(d_out, d_prof, nx, ny, dx);
        std::vector<double> h(n);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(h.data(), d_out, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = FI_E_CUDA;
        } else {
            const double c = 0.25 * (((h[0] + h[n - 1]) + h[(size_t)(ny - 1) * nx]) + h[nx - 1]);
            for (size_t e = 0; e < n; ++e) out[e] = h[e] - c;
        }
    }
    cudaFree(d_edges);
    cudaFree(d_gx);
    cudaFree(d_gw);
    cudaFree(d_prof);
    cudaFree(d_out);
    return rc;
}
