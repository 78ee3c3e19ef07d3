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

// b = (float2)a, elementwise on the device (kernel spectra of the mixed form).
int narrow_spectrum(const double2* a, float2* b, size_t n, cudaStream_t s);

}  // namespace fi
