// fi_init.h — init-time fields computed on the device (fi_init.cu).
#pragma once

#include <cuda_runtime.h>

namespace fi {

// kappa (calc_kappa), GE and GN (elastic and geoid Green's functions) of a
// padded (nx, ny) domain into host arrays; the 42-entry elastic table as the
// single-precision values of the reference.  Returns 0 on success.
int init_fields_device(int nx, int ny, double dx, double dy, double pi_lit, double ge_scale, double g_lit,
                       double r_earth, double m_earth, const float* ge_rn, const float* ge_v, double* kappa,
                       double* GE, double* GN, cudaStream_t s);

// Rheology of the padded domain (isos_init, method-3 branch,
// src/fastisostasy.f90:240-443; src/lv_elva.f90:131-306): lithosphere
// thickness He and rigidity D; for method 3 the layer viscosities lumped to
// eta_eff and the freqdomain factor R, then the viscosity scaling, the
// compressibility factor and the eta_ref transform.  Codes as in fi_params.
struct RheoParams {
    int nx, ny, method;
    int lithosphere, mantle, layering, lumping, nl, visc_scaling_method;
    double zl[8], viscosities[8], dl, E, nu, viscosity_scaling, cc, eta_ref, big_he;
};
// Arrays of a rheology file as its reader returns them (x fastest); a null
// field leaves that part to the codes of RheoParams.
struct RheoFile {
    int nxr, nyr, nzr;
    const double *xr, *yr, *zr;
    const double* thick;      // nxr*nyr lithosphere thickness, before scaling
    double thick_scale;
    const double* log10_eta;  // nxr*nyr*nzr
    const double* stddev;     // nxr*nyr*nzr or null
    int use_stddev;           // viscosity_scaling_method "stddev"
    double smooth_radius;     // rheo_smoothing_radius, 0: none
};
// xc, yc: host coordinates of the padded grid; kappa: host kappa (n).  Any
// output pointer may be null.  Returns 0, or 1 on a CUDA error, 2 on input
// the reference rejects (a smoothing window wider than the grid).
int rheology_device(const RheoParams& P, const double* xc, const double* yc, double dx, const double* kappa,
                    const RheoFile* F, double* He, double* D, double* eta_eff, double* R, cudaStream_t s);

// b = (float2)a, elementwise on the device (kernel spectra of the mixed form).
int narrow_spectrum(const double2* a, float2* b, size_t n, cudaStream_t s);

}  // namespace fi
