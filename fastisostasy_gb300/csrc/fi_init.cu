// fi_init.cu — init-time fields computed on the device.
//
// calc_kappa (src/lv_elva.f90:442-481), the elastic Green's function
// (calc_elastic_green with get_ge_value, src/green_functions.f90:43-91,
// 131-168) and the geoid Green's function (calc_z_ss_green with
// calc_gn_value, :94-128, 171-181) are the cell-by-cell part of isos_init
// that grows with the domain: one thread per cell here instead of a host
// loop, the results copied back for the host-side set-up that follows.
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
    if (cudaMalloc(&buf, 3 * n * sizeof(double)) != cudaSuccess) return 1;
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
    cudaFree(buf);
    if (!rc) kappa[0] = (kappa[nx] + kappa[1]) / 2.0;   // kappa(1,1), src/lv_elva.f90:478
    return rc;
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
