// fi_noalloc.cu — calc_lvelva for callers that cannot allocate device memory.
//
// Some callers may not allocate once they are running: a coupled ice-sheet /
// climate model that divides HBM among its components at start-up and treats
// any later cudaMalloc as a budget violation, or a host loop that must not
// pay the device-wide synchronisation that cudaFree implies.  fi_lvelva needs
// a handle, whose creation allocates, and allocates a temporary on each call.
//
// fi_lvelva_static runs the same FP64 viscous-rate kernels on device arrays
// owned by the caller and allocates nothing.  Its scratch (load term,
// 1/(2 eta), the stencil output, the half spectrum, the 1/(kappa R)
// multipliers, the twiddle tables and the raw inverse-transform output) lives
// in one file-scope __device__ array sized for grids of at most
// FI_STATIC_MAX_N x FI_STATIC_MAX_N cells (256 x 256: 3,219,472 bytes), which
// every GPU that loads the library holds until the process exits.  Larger or
// odd-sized grids are refused with FI_E_SIZE before any work is queued.
// Nothing in the scratch has to start at zero: every word a kernel reads was
// written earlier in the same call.
//
// Host code cannot use the array's name as a device address, so every call
// looks the address up on the current device with cudaGetSymbolAddress (a
// lookup that allocates nothing once the library's device code is loaded,
// and that stays valid after a cudaDeviceReset, which a cached pointer would
// not).  The first call on a device loads that code; make it before
// capturing any stream.  All calls on one device share the one array: calls
// whose work can overlap on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.
//
// Spacing: dx, dy for a uniform grid, or the per-cell dx*K and dy*K fields
// of a distorted projection (src/fastisostasy.f90:152-155), which
// calc_lvelva's finite differences use cell by cell (src/lv_elva.f90:31).
#include <cmath>
#include <cstring>

#include "../../include/fi_gpu.h"
#include "fi_kernels.h"
#include "fi_state.h"

using namespace fi;

namespace {

constexpr int NA_N = FI_STATIC_MAX_N;                       // max cells per axis
constexpr int NA_CELLS = NA_N * NA_N;
constexpr int NA_SP = ((NA_N / 2 + 1) + 7) / 8 * 8;          // spectrum row pitch (complex)
constexpr size_t NA_SPEC = (size_t)NA_N * NA_SP;             // spectrum entries

// byte layout of the scratch array
constexpr size_t OFF_Q0 = 0;
constexpr size_t OFF_I2E = OFF_Q0 + (size_t)NA_CELLS * 8;
constexpr size_t OFF_F = OFF_I2E + (size_t)NA_CELLS * 8;
constexpr size_t OFF_RAW = OFF_F + (size_t)NA_CELLS * 8;
constexpr size_t OFF_S = OFF_RAW + (size_t)NA_CELLS * 8;
constexpr size_t OFF_MA = OFF_S + NA_SPEC * 16;
constexpr size_t OFF_MB = OFF_MA + NA_SPEC * 8;
constexpr size_t OFF_TWR = OFF_MB + NA_SPEC * 8;             // row FFT, length nx/2
constexpr size_t OFF_TWC = OFF_TWR + (size_t)(NA_N / 2) * 16; // column FFT, length ny
constexpr size_t OFF_RTW = OFF_TWC + (size_t)NA_N * 16;       // real-FFT twiddles, nx/2 + 1
constexpr size_t NA_BYTES = OFF_RTW + (size_t)(NA_N / 2 + 1) * 16;
static_assert(NA_BYTES == 3219472, "scratch size stated in the header comment");

static __device__ __align__(256) unsigned char g_fi_static_scratch[NA_BYTES];

// exp(-2 pi i t / n) for t < n, and exp(-2 pi i k / nx) for k <= nx/2
__global__ void k_na_twiddles(double2* twr, int nr, double2* twc, int nc, double2* rtw, int nx)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double s, c;
    if (t < nr) { sincospi(-2.0 * t / nr, &s, &c); twr[t] = make_double2(c, s); }
    if (t < nc) { sincospi(-2.0 * t / nc, &s, &c); twc[t] = make_double2(c, s); }
    if (t <= nx / 2) { sincospi(-2.0 * t / nx, &s, &c); rtw[t] = make_double2(c, s); }
}

// load term, 1/(2 eta) and the multipliers m(k, l), m(-k, l) in the half-spectrum layout
__global__ void k_na_fields(const double* __restrict__ cf, const uint8_t* __restrict__ mask,
                            const double* __restrict__ eta, const double* __restrict__ kappa,
                            const double* __restrict__ R, double g, int nx, int ny, int sp, double* q0,
                            double* i2e, double* mA, double* mB)
{
    const size_t n = (size_t)nx * ny;
    const int h = nx / 2;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        q0[e] = mask[e] ? -g * cf[e] : 0.0;
        i2e[e] = 1.0 / (2.0 * eta[e]);
        const int i = (int)(e % nx), l = (int)(e / nx);
        if (i <= h) {
            const size_t a = (size_t)l * nx + i, b = (size_t)l * nx + (nx - i) % nx;
            mA[(size_t)l * sp + i] = 1.0 / (kappa[a] * R[a]);
            mB[(size_t)l * sp + i] = 1.0 / (kappa[b] * R[b]);
        }
    }
}

FftDesc na_factorize(int n)
{
    FftDesc d;
    memset(&d, 0, sizeof(d));
    d.n = n;
    int m = n, e2 = 0;
    while (m % 2 == 0) { m /= 2; e2++; }
    int n8 = e2 / 3, r = e2 % 3, n4 = 0, n2 = 0;
    if (r == 1) { if (n8 > 0) { n8--; n4 = 2; } else n2 = 1; }
    else if (r == 2) n4 = 1;
    for (int i = 0; i < n8; ++i) d.fac[d.nf++] = 8;
    for (int i = 0; i < n4; ++i) d.fac[d.nf++] = 4;
    for (int i = 0; i < n2; ++i) d.fac[d.nf++] = 2;
    for (int f = 3; m > 1; f += 2)
        while (m % f == 0) { d.fac[d.nf++] = f; m /= f; }
    return d;
}

}  // namespace

extern "C" int fi_lvelva_static(const double* d_w, const double* d_canom_full, const uint8_t* d_maskactive,
                                const double* d_D_lith, const double* d_eta_eff, const double* d_kappa,
                                const double* d_R, const double* d_dx_matrix, const double* d_dy_matrix, int nx,
                                int ny, double dx, double dy, double g, double nu, double sec_per_year,
                                double* d_dwdt, void* stream)
{
    if (!d_w || !d_canom_full || !d_maskactive || !d_D_lith || !d_eta_eff || !d_kappa || !d_R || !d_dwdt)
        return FI_E_ARG;
    if (!(dx > 0.0) || !(dy > 0.0)) return FI_E_ARG;
    if ((d_dx_matrix == nullptr) != (d_dy_matrix == nullptr)) return FI_E_ARG;   // both or neither
    // grids the static scratch cannot hold are refused, not truncated
    if (nx < 4 || ny < 4 || nx > NA_N || ny > NA_N || (nx & 1) || (ny & 1)) return FI_E_SIZE;
    cudaStream_t s = (cudaStream_t)stream;
    void* sym = nullptr;
    if (cudaGetSymbolAddress(&sym, g_fi_static_scratch) != cudaSuccess || !sym) return FI_E_CUDA;
    unsigned char* const base = static_cast<unsigned char*>(sym);
    double* q0 = reinterpret_cast<double*>(base + OFF_Q0);
    double* i2e = reinterpret_cast<double*>(base + OFF_I2E);
    double* f = reinterpret_cast<double*>(base + OFF_F);
    double* raw = reinterpret_cast<double*>(base + OFF_RAW);
    double2* S = reinterpret_cast<double2*>(base + OFF_S);
    double* mA = reinterpret_cast<double*>(base + OFF_MA);
    double* mB = reinterpret_cast<double*>(base + OFF_MB);
    double2* twr = reinterpret_cast<double2*>(base + OFF_TWR);
    double2* twc = reinterpret_cast<double2*>(base + OFF_TWC);
    double2* rtw = reinterpret_cast<double2*>(base + OFF_RTW);

    Plan2D p;
    memset(&p, 0, sizeof(p));
    p.nx = nx;
    p.ny = ny;
    p.h = nx / 2;
    p.sp = ((p.h + 1) + 7) / 8 * 8;
    p.row.d = na_factorize(p.h);
    p.row.tw64 = twr;
    p.col.d = na_factorize(ny);
    p.col.tw64 = twc;
    p.rtw64 = rtw;

    const int nt = ny > nx / 2 + 1 ? ny : nx / 2 + 1;
    k_na_twiddles<<<(nt + 255) / 256, 256, 0, s>>>(twr, p.h, twc, ny, rtw, nx);
    k_na_fields<<<(int)(((size_t)nx * ny + 255) / 256), 256, 0, s>>>(d_canom_full, d_maskactive, d_eta_eff, d_kappa,
                                                                     d_R, g, nx, ny, p.sp, q0, i2e, mA, mB);
    FlexCoef c;
    memset(&c, 0, sizeof(c));
    c.nu = nu;
    c.one_minus_nu = 1.0 - nu;
    c.inv_dx = 1.0 / dx;
    c.inv_2dx = 1.0 / (2 * dx);
    c.inv_dx2 = 1.0 / (dx * dx);
    c.inv_dy = 1.0 / dy;
    c.inv_2dy = 1.0 / (2 * dy);
    c.inv_dy2 = 1.0 / (dy * dy);
    c.dxm = d_dx_matrix;   // null: uniform spacing from dx, dy
    c.dym = d_dy_matrix;
    launch_flexure<double>(d_w, nullptr, q0, d_maskactive, d_D_lith, i2e, f, nx, ny, c, s);
    launch_rows_fwd<double>(f, nx, nx, ny, S, p, s);
    launch_cols_hartley<double>(S, mA, mB, 0, p, s);
    const double norm = (double)(float)((long long)nx * ny);   // nx*ny*1. (default real)
    launch_rows_inv<double>(S, raw, p, 1.0 / norm, s);
    rhs_finish<double>(d_dwdt, raw, nx, ny, sec_per_year, s);
    return cudaGetLastError() == cudaSuccess ? FI_OK : FI_E_CUDA;
}
