// fi_batch.h — batched launches over the members of an ensemble.
//
// A batched launch runs one pass of the reference-compatible Tsit5 attempt
// (flexure stencil, row rFFT, Hartley column pass, inverse row rFFT, the two
// error-norm reductions, the state commit) for every member of an ensemble
// in a single kernel launch: member m owns the blocks [off[m], off[m+1]) and
// runs exactly the blocks its own single-domain launch would run, so every
// member gets the bits it gets alone.  Members may differ in size.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fi_common.cuh"
#include "fi_kernels.h"
#include "fi_state.h"

namespace fi {

struct BMember {
    Plan2D p;                 // RHS transform plan
    FlexCoef fc;              // flexure coefficients
    FlexCoefF fcf;            // the same in float (mixed form)
    const double* y;          // the RHS is evaluated at now%w
    const void* q0;           // load term (T)
    const uint8_t* mask;
    const void* D;            // rigidity (T)
    const void* inv2eta;      // 1/(2 eta) (T)
    void* f;                  // flexure output (T)
    void* S;                  // half spectrum (T complex)
    const void* mA;           // 1/(kappa R) at (k, l), (-k, l) (T)
    const void* mB;
    void* raw;                // RHS output (T)
    void* raw7[7];            // true stages: the seven stage outputs (T); raw7[0] = raw
    double* yst;              // true stages: stage state buffer (stages 1-5; stage 6 is d.ts_x2)
    const double* wref;       // true stages: w_ref of the mantle term
    // true stages, mixed form (null otherwise): the float pair of x with
    // dxw = (x - w_ref) of the pairs, the stage state's pair and dxw, and
    // the pair of w_ref
    float *xhi, *xlo, *xdw, *yhi, *ylo, *ydw;
    const float *wrhi, *wrlo;
    int even;
    int RB, CB;               // rows per row block, columns per column block
    int fgx;                  // flexure blocks along x (FP64 tiles)
    int fseg;                 // output rows per flexure warp task (mixed column strips)
    int red_nblk;             // blocks of the reduction kernels
    double norm_scale;        // 1 / (nx*ny*1.) as the reference normalises
    float norm_scale_f;       // the same in float: no FP64 division per thread
    Dom d;
    double atol, rtol, q, dt_max;
};

// per-update scalars of one member (k_set_args)
struct BArgs {
    Ctl* ctl;
    double tf, bsl, A_ocean;
    int method, write_bsl;
};

// Members with work in the current attempt, compacted by the attempt-begin
// kernel: ids[j] for j < *cnt, member ids[j] owning the virtual blocks
// [coff[j], coff[j+1]) of a batched launch.  Seven lists share one int
// buffer of blist_ints(nm) entries: 0 flexure, 1 row transforms, 2 column
// transforms (members that need a new RHS), 3 attempt kernels, 4 flexure,
// 5 row transforms, 6 column transforms (members with an attempt left; the
// RHS of true stages 1-6).
struct BList {
    const int* ids;
    const int* coff;
    const int* cnt;
};
inline size_t blist_ints(int nm) { return 2 + 2 * (size_t)nm + 7 * ((size_t)nm + 1); }
inline BList blist(const int* base, int nm, int kind)
{
    BList L;
    L.cnt = base + (kind >= 3 ? 1 : 0);
    L.ids = base + 2 + (kind >= 3 ? nm : 0);
    L.coff = base + 2 + 2 * (size_t)nm + (size_t)kind * (nm + 1);
    return L;
}

// Virtual blocks of the mixed batched flexure (8 column-strip warp tasks each).
int batch_flexure_blocks(int nx, int ny, int seg);

// Block shapes of the single-domain launches (shared with the batched ones).
int rhs_rows_per_block(int h);
int rhs_threads_for(int work);
template <typename T> int rhs_cols_per_block(int ny);
int reduce_grid(size_t n);
int ts_grid(size_t n);           // blocks of the Tsit5 attempt reductions

// Raise the shared-memory limits of the batched transform kernels (before
// any capture).
template <typename T> void batch_prepare(size_t rows_smem, size_t cols_smem);

// Resident blocks per SM of the batched reduction kernels.
template <typename T> int batch_red_resident();
// Resident grid sizes of the batched kernels (blocks per launch).
template <typename T> void batch_grids(size_t rows_smem, size_t cols_smem, int rows_threads, int cols_threads,
                                       int* g_flex, int* g_rows, int* g_cols, int* g_red);

// Phase kernels over all members; nblk is the launch's (resident) grid.
template <typename T> void batch_flexure(const BMember* M, BList L, int nblk, cudaStream_t s);
template <typename T>
void batch_rows_fwd(const BMember* M, BList L, int nblk, int threads, size_t smem, cudaStream_t s);
template <typename T>
void batch_cols_hartley(const BMember* M, BList L, int nblk, int threads, size_t smem, cudaStream_t s);
template <typename T>
void batch_rows_inv(const BMember* M, BList L, int nblk, int threads, size_t smem, cudaStream_t s, int stage = 0);
template <typename T> void batch_ts_max(const BMember* M, BList L, int nblk, cudaStream_t s);
template <typename T>
void batch_ts_err(const BMember* M, BList L, int nblk, cudaStream_t s);
template <typename T> void batch_ts_commit(const BMember* M, BList L, int nblk, cudaStream_t s);
// true stages (Dormand-Prince 5(4) with FSAL) per member
template <typename T> void batch_dp_stage(const BMember* M, BList L, int nblk, int i, cudaStream_t s);
template <typename T> void batch_dp_err(const BMember* M, BList L, int nblk, cudaStream_t s);
template <typename T> void batch_fsal(const BMember* M, BList L, int nblk, cudaStream_t s);
template <typename T> void batch_flexure_y(const BMember* M, BList L, int nblk, int stage, cudaStream_t s);
// mixed form with the float pair of now%w: ts_fused / ts_commit_pair per member
void batch_ts_fused(const BMember* M, BList L, int nblk, cudaStream_t s);
void batch_ts_commit_pair(const BMember* M, BList L, int nblk, cudaStream_t s);
void batch_loop_begin(const BMember* M, int nm, cudaStream_t s);
// attempt_begin of every member, then the compacted lists (cl, blist_ints(nm)
// ints) from the members' static block offsets (off, 4 x (nm + 1)).
void batch_attempt_begin(const BMember* M, int nm, int max_iter, const int* off, int* cl, cudaStream_t s);
// more_out == NULL: sets the WHILE condition `loop`; else writes it there
void batch_attempt_end(const BMember* M, int nm, cudaGraphConditionalHandle loop, cudaStream_t s,
                       int* more_out = nullptr, int fsal = 0);
void batch_set_args(const BArgs* a, int nm, cudaStream_t s);

// member owning global block b of a batched launch (off has nm + 1 entries)
__device__ __forceinline__ int batch_member(const int* __restrict__ off, int nm, int b)
{
    int lo = 0, hi = nm - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Grid-stride walk over the virtual blocks of the listed members: fn(m,
// local block) runs for each, skipped where active(m) is false (uniform over
// the block; a member without work is skipped in one jump).  Launches size
// their grid to what stays resident, not to the members' total block count,
// and members without work cost nothing.
template <typename Act, typename Fn>
__device__ __forceinline__ void batch_walk(BList L, Act active, Fn fn)
{
    const int na = __ldg(L.cnt);
    if (na <= 0) return;
    const int total = __ldg(L.coff + na);
    const int stride = (int)gridDim.x;
    int vb = (int)blockIdx.x;
    if (vb >= total) return;
    int j = batch_member(L.coff, na, vb);
    while (vb < total) {
        while (__ldg(L.coff + j + 1) <= vb) ++j;
        const int m = __ldg(L.ids + j);
        const int end = __ldg(L.coff + j + 1);
        if (!active(m)) {
            vb += ((end - vb + stride - 1) / stride) * stride;
            continue;
        }
        fn(m, vb - __ldg(L.coff + j));
        vb += stride;
    }
}

}  // namespace fi
