// fi_fft.cuh — block-cooperative shared-memory Stockham FFT (any length).
//
// Self-sorting Stockham formulation: a stage of radix R over sub-transform
// size Ns takes butterfly j from x[j + r*n/R] (r < R), multiplies by the
// twiddle w^((j mod Ns) * r * n/(Ns*R)) with w = exp(-2 pi i / n), does a
// radix-R DFT and writes y[(j/Ns)*Ns*R + j mod Ns + r*Ns].  After all stages
// the result is in natural order.  All threads of the block walk over the
// butterflies of `nl` lines (line l at offset l*ls), so a block can work on
// several rows or columns at once; every stage ends in __syncthreads().
//
// Twiddles come from a per-length table tw[t] = exp(-2 pi i t / n) built on
// the host in long double; sign = -1 is the forward transform, +1 the
// unnormalised inverse.  SH = true reads the table from a shared-memory copy
// (a persistent kernel keeps it resident instead of refetching it from L2
// after the data it streams has pushed it out of L1).
#pragma once

#include "fi_common.cuh"

namespace fi {

template <typename T, typename C2, bool SH = false>
__device__ __forceinline__ C2 tw_load(const C2* __restrict__ tw, int t, int sign)
{
    C2 w = SH ? tw[t] : __ldg(tw + t);
    if (sign > 0) w.y = -w.y;
    return w;
}

// radix-2/4/8 DFTs in registers
template <typename T, typename C2>
__device__ __forceinline__ void dft2(C2& a, C2& b)
{
    C2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

// multiply by -i (forward) or +i (inverse)
template <typename C2>
__device__ __forceinline__ C2 mul_mi(C2 a, int sign)
{
    C2 r;
    if (sign < 0) { r.x = a.y; r.y = -a.x; }
    else { r.x = -a.y; r.y = a.x; }
    return r;
}

template <typename T, typename C2>
__device__ __forceinline__ void dft4(C2& v0, C2& v1, C2& v2, C2& v3, int sign)
{
    C2 s0 = cadd(v0, v2), d0 = csub(v0, v2);
    C2 s1 = cadd(v1, v3), d1 = mul_mi(csub(v1, v3), sign);
    v0 = cadd(s0, s1);
    v2 = csub(s0, s1);
    v1 = cadd(d0, d1);
    v3 = csub(d0, d1);
}

template <typename T, typename C2>
__device__ __forceinline__ void dft8(C2* v, int sign)
{
    // even / odd radix-4, then combine with w8^q
    C2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<T, C2>(e0, e1, e2, e3, sign);
    dft4<T, C2>(o0, o1, o2, o3, sign);
    const T h = (T)0.70710678118654752440084436210484903928;
    // o1 *= w8^1, o2 *= w8^2, o3 *= w8^3 ; w8 = exp(sign * i pi / 4)
    C2 t1, t3;
    if (sign < 0) {
        t1.x = h * (o1.x + o1.y); t1.y = h * (o1.y - o1.x);     // (1 - i)/sqrt2
        t3.x = h * (o3.y - o3.x); t3.y = -h * (o3.x + o3.y);    // (-1 - i)/sqrt2
    } else {
        t1.x = h * (o1.x - o1.y); t1.y = h * (o1.y + o1.x);     // (1 + i)/sqrt2
        t3.x = -h * (o3.x + o3.y); t3.y = h * (o3.x - o3.y);    // (-1 + i)/sqrt2
    }
    C2 t2 = mul_mi(o2, sign);
    v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
    v[1] = cadd(e1, t1); v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2); v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3); v[7] = csub(e3, t3);
}

template <typename T, typename C2>
__device__ __forceinline__ void dft3(C2& a, C2& b, C2& c, int sign)
{
    const T c1 = (T)-0.5;
    const T s1 = (T)(sign < 0 ? -0.86602540378443864676372317075293618 : 0.86602540378443864676372317075293618);
    C2 s = cadd(b, c), d = csub(b, c);
    C2 m;
    m.x = a.x + c1 * s.x;
    m.y = a.y + c1 * s.y;
    a = cadd(a, s);
    // +/- i*s1*d
    C2 r;
    r.x = -s1 * d.y;
    r.y = s1 * d.x;
    b = cadd(m, r);
    c = csub(m, r);
}

// One line-parallel Stockham stage.  Specialised radices keep the R values
// in registers; other radices use a direct sum over the table.
// Index modes of a stage: FFT_ANY divides by the stage's runtime sizes,
// FFT_AUTO takes shifts and masks when the length is a power of two and
// divides otherwise, FFT_POW2 handles power-of-two lengths only (one loop,
// radices 8, 4, 2: the smallest code, for the persistent step engine).
enum { FFT_ANY = 0, FFT_AUTO = 1, FFT_POW2 = 2 };

template <typename T, int R, bool SH = false, int MODE = FFT_AUTO>
__device__ __forceinline__ void stage_fixed(const typename vec2<T>::type* __restrict__ src,
                                            typename vec2<T>::type* __restrict__ dst, int n, int nl,
                                            int ls, int Ns, const typename vec2<T>::type* __restrict__ tw,
                                            int sign, int tid, int nthr)
{
    typedef typename vec2<T>::type C2;
    const int NR = n / R;
    const int tstep = n / (Ns * R);
    const int items = nl * NR;
    auto butterfly = [&](int line, int j, int jm, int out0) {
        const C2* x = src + (size_t)line * ls;
        C2* y = dst + (size_t)line * ls;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 a = x[j + r * NR];
            if (r > 0 && jm > 0) a = cmul(a, tw_load<T, C2, SH>(tw, jm * r * tstep, sign));
            v[r] = a;
        }
        if (R == 2) dft2<T, C2>(v[0], v[1]);
        else if (R == 4) dft4<T, C2>(v[0], v[1], v[2], v[3], sign);
        else if (R == 8) dft8<T, C2>(v, sign);
        else if (R == 3) dft3<T, C2>(v[0], v[1], v[2], sign);
#pragma unroll
        for (int r = 0; r < R; ++r) y[out0 + r * Ns] = v[r];
    };
    if (MODE == FFT_POW2 || (MODE == FFT_AUTO && (n & (n - 1)) == 0 && (R & (R - 1)) == 0)) {
        // power-of-two length: NR and Ns are powers of two, so the butterfly
        // index splits by shifts and masks instead of three runtime integer
        // divisions per butterfly (long instruction sequences on the
        // critical path of a stage that only a few warps execute)
        const int lnr = __ffs(NR) - 1, lns = __ffs(Ns) - 1, lr = __ffs(R) - 1;
        for (int it = tid; it < items; it += nthr) {
            const int line = it >> lnr;
            const int j = it & (NR - 1);
            const int jm = j & (Ns - 1);
            butterfly(line, j, jm, ((j >> lns) << (lns + lr)) + jm);
        }
        return;
    }
    if constexpr (MODE != FFT_POW2) {
        for (int it = tid; it < items; it += nthr) {
            const int line = it / NR;
            const int j = it - line * NR;
            const int jm = j % Ns;
            butterfly(line, j, jm, (j / Ns) * Ns * R + jm);
        }
    }
}

template <typename T, bool SH = false>
__device__ void stage_generic(const typename vec2<T>::type* __restrict__ src,
                              typename vec2<T>::type* __restrict__ dst, int n, int nl, int ls, int R,
                              int Ns, const typename vec2<T>::type* __restrict__ tw, int sign, int tid,
                              int nthr)
{
    typedef typename vec2<T>::type C2;
    const int NR = n / R;
    const int tstep = n / (Ns * R);
    const int step = n / R;   // table stride of the R-th roots of unity
    const int items = nl * NR * R;
    for (int it = tid; it < items; it += nthr) {
        const int q = it % R;
        const int jl = it / R;
        const int line = jl / NR;
        const int j = jl - line * NR;
        const C2* x = src + (size_t)line * ls;
        C2* y = dst + (size_t)line * ls;
        const int jm = j % Ns;
        const int out0 = (j / Ns) * Ns * R + jm;
        C2 acc = mk2<T>((T)0, (T)0);
        for (int r = 0; r < R; ++r) {
            C2 a = x[j + r * NR];
            if (r > 0 && jm > 0) a = cmul(a, tw_load<T, C2, SH>(tw, jm * r * tstep, sign));
            const int e = ((r * q) % R) * step;
            acc = cadd(acc, cmul(a, tw_load<T, C2, SH>(tw, e, sign)));
        }
        y[out0 + q * Ns] = acc;
    }
}

// Runs all stages on nl lines held in buf0 (scratch buf1, same shape).
// Returns the buffer holding the result.  Must be called by every thread of
// the block (it synchronises internally); the caller synchronises before.
// MODE: see stage_fixed.  The persistent step engine inlines four
// transforms; carrying both loop forms in each made it slower (1.20 -> 1.24
// ms per 512^2 update) where the per-launch transform kernels gained up to
// 5 %, so the engine takes FFT_POW2 or FFT_ANY by its plan.
template <typename T, bool SH = false, int MODE = FFT_AUTO>
__device__ typename vec2<T>::type* block_fft(typename vec2<T>::type* buf0, typename vec2<T>::type* buf1,
                                             const FftDesc& d, int nl, int ls,
                                             const typename vec2<T>::type* __restrict__ tw, int sign)
{
    typedef typename vec2<T>::type C2;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    C2* src = buf0;
    C2* dst = buf1;
    int Ns = 1;
    for (int s = 0; s < d.nf; ++s) {
        const int R = d.fac[s];
        switch (R) {
        case 8: stage_fixed<T, 8, SH, MODE>(src, dst, d.n, nl, ls, Ns, tw, sign, tid, nthr); break;
        case 4: stage_fixed<T, 4, SH, MODE>(src, dst, d.n, nl, ls, Ns, tw, sign, tid, nthr); break;
        case 2: stage_fixed<T, 2, SH, MODE>(src, dst, d.n, nl, ls, Ns, tw, sign, tid, nthr); break;
        case 3:
            if constexpr (MODE != FFT_POW2) stage_fixed<T, 3, SH, MODE>(src, dst, d.n, nl, ls, Ns, tw, sign, tid, nthr);
            break;
        default:
            if constexpr (MODE != FFT_POW2) stage_generic<T, SH>(src, dst, d.n, nl, ls, R, Ns, tw, sign, tid, nthr);
            break;
        }
        __syncthreads();
        C2* t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    return src;
}

}  // namespace fi
