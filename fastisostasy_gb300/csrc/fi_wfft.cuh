// fi_wfft.cuh — warp-level complex FFT of length n = 32 * P (P = 1..32).
//
// Four-step split n = P x 32: lane L holds x[L + 32 p] (p < P) in registers;
//   1. P-point DFT over the registers           (natural order, in registers)
//   2. twiddle by w_n^(L k1)
//   3. 32-point DFT across the lanes: five radix-2 decimation-in-frequency
//      stages on __shfl_xor_sync pairs (output in bit-reversed lane order)
// so that afterwards lane L, register k1 holds X[k1 + P * brev5(L)].
// No shared memory and no block barrier: a warp transforms its line alone.
// Twiddles come from the per-length table tw[t] = exp(-2 pi i t / n).
#pragma once

#include "fi_fft.cuh"

namespace fi {

__device__ __forceinline__ int brev5(int x) { return __brev((unsigned)x) >> 27; }

// w_32^m for m < 32 (double), broadcast reads with compile-time indices
__constant__ double2 c_w32d[32] = {
    {1.0, 0.0},
    {0.98078528040323043, -0.19509032201612825},
    {0.92387953251128674, -0.38268343236508978},
    {0.83146961230254524, -0.55557023301960218},
    {0.70710678118654757, -0.70710678118654757},
    {0.55557023301960218, -0.83146961230254524},
    {0.38268343236508978, -0.92387953251128674},
    {0.19509032201612825, -0.98078528040323043},
    {0.0, -1.0},
    {-0.19509032201612825, -0.98078528040323043},
    {-0.38268343236508978, -0.92387953251128674},
    {-0.55557023301960218, -0.83146961230254524},
    {-0.70710678118654757, -0.70710678118654757},
    {-0.83146961230254524, -0.55557023301960218},
    {-0.92387953251128674, -0.38268343236508978},
    {-0.98078528040323043, -0.19509032201612825},
    {-1.0, 0.0},
    {-0.98078528040323043, 0.19509032201612825},
    {-0.92387953251128674, 0.38268343236508978},
    {-0.83146961230254524, 0.55557023301960218},
    {-0.70710678118654757, 0.70710678118654757},
    {-0.55557023301960218, 0.83146961230254524},
    {-0.38268343236508978, 0.92387953251128674},
    {-0.19509032201612825, 0.98078528040323043},
    {0.0, 1.0},
    {0.19509032201612825, 0.98078528040323043},
    {0.38268343236508978, 0.92387953251128674},
    {0.55557023301960218, 0.83146961230254524},
    {0.70710678118654757, 0.70710678118654757},
    {0.83146961230254524, 0.55557023301960218},
    {0.92387953251128674, 0.38268343236508978},
    {0.98078528040323043, 0.19509032201612825},
};

template <typename T, typename C2>
__device__ __forceinline__ C2 w32c(int m, int sign)
{
    const double2 w = c_w32d[m & 31];
    C2 r;
    r.x = (T)w.x;
    r.y = (T)(sign > 0 ? -w.y : w.y);
    return r;
}

// P-point DFT of registers v[0..P), natural-order output.
template <typename T, int P> struct RegDft;

template <typename T> struct RegDft<T, 1> {
    template <typename C2> __device__ __forceinline__ static void run(C2*, int) {}
};
template <typename T> struct RegDft<T, 2> {
    template <typename C2> __device__ __forceinline__ static void run(C2* v, int) { dft2<T, C2>(v[0], v[1]); }
};
template <typename T> struct RegDft<T, 4> {
    template <typename C2> __device__ __forceinline__ static void run(C2* v, int s) { dft4<T, C2>(v[0], v[1], v[2], v[3], s); }
};
template <typename T> struct RegDft<T, 8> {
    template <typename C2> __device__ __forceinline__ static void run(C2* v, int s) { dft8<T, C2>(v, s); }
};
// 16 = 4 x 4 and 32 = 8 x 4:  X[k1 + Q k2] = sum_n2 w^(n2 k1) [sum_n1 x[n2 + 4 n1] w_Q^(n1 k1)] w_4^(n2 k2)
template <typename T> struct RegDft<T, 16> {
    template <typename C2> __device__ __forceinline__ static void run(C2* v, int s)
    {
        C2 y[4][4];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            C2 a0 = v[n2], a1 = v[n2 + 4], a2 = v[n2 + 8], a3 = v[n2 + 12];
            dft4<T, C2>(a0, a1, a2, a3, s);
            y[n2][0] = a0;
            y[n2][1] = cmul(a1, w32c<T, C2>(2 * n2 * 1, s));
            y[n2][2] = cmul(a2, w32c<T, C2>(2 * n2 * 2, s));
            y[n2][3] = cmul(a3, w32c<T, C2>(2 * n2 * 3, s));
        }
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            C2 b0 = y[0][k1], b1 = y[1][k1], b2 = y[2][k1], b3 = y[3][k1];
            dft4<T, C2>(b0, b1, b2, b3, s);
            v[k1] = b0;
            v[k1 + 4] = b1;
            v[k1 + 8] = b2;
            v[k1 + 12] = b3;
        }
    }
};
template <typename T> struct RegDft<T, 32> {
    template <typename C2> __device__ __forceinline__ static void run(C2* v, int s)
    {
        C2 y[4][8];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            C2 a[8];
#pragma unroll
            for (int n1 = 0; n1 < 8; ++n1) a[n1] = v[n2 + 4 * n1];
            dft8<T, C2>(a, s);
#pragma unroll
            for (int k1 = 0; k1 < 8; ++k1) y[n2][k1] = k1 == 0 ? a[0] : cmul(a[k1], w32c<T, C2>(n2 * k1, s));
        }
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) {
            C2 b0 = y[0][k1], b1 = y[1][k1], b2 = y[2][k1], b3 = y[3][k1];
            dft4<T, C2>(b0, b1, b2, b3, s);
            v[k1] = b0;
            v[k1 + 8] = b1;
            v[k1 + 16] = b2;
            v[k1 + 24] = b3;
        }
    }
};

template <typename C2> __device__ __forceinline__ C2 shfl_xor_c(C2 a, int d)
{
    C2 r;
    r.x = __shfl_xor_sync(0xffffffffu, a.x, d);
    r.y = __shfl_xor_sync(0xffffffffu, a.y, d);
    return r;
}

// In place on v[P] (input x[lane + 32 p]); output v[k1] = X[k1 + P brev5(lane)].
template <typename T, int P>
__device__ __forceinline__ void warp_fft(typename vec2<T>::type (&v)[P], int lane,
                                         const typename vec2<T>::type* __restrict__ tw, int sign)
{
    typedef typename vec2<T>::type C2;
    constexpr int n = 32 * P;
    // all twiddles of this lane first, so their loads overlap
    C2 w2[P > 1 ? P - 1 : 1], w3[5];
#pragma unroll
    for (int k1 = 1; k1 < P; ++k1) w2[k1 - 1] = tw_load<T, C2>(tw, lane * k1, sign);
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        const int d = 16 >> s;
        w3[s] = tw_load<T, C2>(tw, (lane & (d - 1)) * (16 / d) * (n / 32), sign);
    }
    RegDft<T, P>::run(v, sign);
#pragma unroll
    for (int k1 = 1; k1 < P; ++k1) v[k1] = cmul(v[k1], w2[k1 - 1]);
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        const int d = 16 >> s;
        const C2 w = w3[s];
        const bool upper = (lane & d) == 0;
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            const C2 o = shfl_xor_c(v[k1], d);
            v[k1] = upper ? cadd(v[k1], o) : cmul(csub(o, v[k1]), w);
        }
    }
}

}  // namespace fi
