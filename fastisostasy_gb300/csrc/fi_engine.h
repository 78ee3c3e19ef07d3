// fi_engine.h — the persistent cooperative RK4 step engine (fi_engine.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fi_common.cuh"
#include "fi_kernels.h"

namespace fi {

struct EngineArgs {
    Plan2D p;
    FlexCoef fc;                     // uniform spacing only
    FlexCoefF fcf;                   // the same in float (mixed form: no per-thread conversions)
    double* x;                       // integrator state (double)
    double* w;                       // now%w
    float* xhi;                      // mixed form: x = xhi + xlo
    float* xlo;
    const float* wrefhi;             // mixed form: w_ref = wrefhi + wreflo
    const float* wreflo;
    const double* wref;              // plain form
    const void* q0;                  // RHS load term, field type
    const void* D;
    const void* inv2eta;
    const void* mA;                  // 1/(kappa R) factors, column-major (k*ny + l)
    const void* mB;
    int even;
    const uint8_t* mask;
    void* raw[4];                    // stage outputs, field type
    void* S;                         // half spectrum, field type complex, row-major (pitch p.sp)
    void* ST;                        // the same, column-major (k*ny + l): phase A -> phase B
    Ctl* ctl;
    int nsteps;
    int CB;                          // spectrum columns per phase-B item
    int ra;                          // rows per stencil item (kernel shape: 2 or 4)
    int p2;                          // both transform lengths are powers of two
    double spy;
    double norm_scale;               // 1 / (nx*ny*1.) as the reference normalises
    float norm_scale_f;              // the same in float
    unsigned long long* trace;       // optional: %globaltimer at phase boundaries of the first step
    unsigned* bar;                   // grid-barrier arrival counter, zeroed before the launch
    int bar_phantom;                 // test only: arrivals expected beyond the grid (a wait that expires)

    template <typename T> __device__ __forceinline__ const T* q0_T() const { return (const T*)q0; }
    template <typename T> __device__ __forceinline__ const T* D_T() const { return (const T*)D; }
    template <typename T> __device__ __forceinline__ const T* inv2eta_T() const { return (const T*)inv2eta; }
    template <typename T> __device__ __forceinline__ const T* mA_T() const { return (const T*)mA; }
    template <typename T> __device__ __forceinline__ const T* mB_T() const { return (const T*)mB; }
};

// Grid size (co-resident blocks), phase-B column count, dynamic shared
// memory, rows per stencil item and transform index mode of the engine for
// this transform plan; 0 if it cannot run.
template <typename T> int engine_config(const Plan2D& p, int* grid, int* CB, size_t* smem, int* RA, int* P2);
template <typename T> cudaError_t engine_launch(const EngineArgs& g, int grid, size_t smem, cudaStream_t s);
void split_hilo(const double* x, float* hi, float* lo, size_t n, cudaStream_t s);
// split plus dxw = (hi - wrhi) + (lo - wrlo) (the kernel sequence's mixed RK4 stages)
void split_hilo_dxw(const double* x, float* hi, float* lo, const float* wrhi, const float* wrlo, float* dxw, size_t n,
                    cudaStream_t s);

}  // namespace fi
