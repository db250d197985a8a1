// fft_reg.cuh -- in-register DFTs and the two-phase ("four-step") line FFT used
// by the register convolution passes.
//
// A line of length n = N1*N2 (index j = w + N1*j2) is transformed by N1
// workers.  Phase 1: worker w holds x[w + N1*j2], j2 < N2, does a DFT of size
// N2 in registers and multiplies by the twiddle W_n^(w*k2).  The values are
// exchanged through shared memory so that worker k2 (< N2) holds the N1 values
// of column k2; phase 2 is a DFT of size N1 in registers, giving
// X[k2 + N2*k1] in register k1.  Forward = exp(-2 pi i jk/n) (FFTW sign).
#pragma once
#include "fft.cuh"

namespace fansgpu {

template <typename T, int M, bool INV>
struct Dft;

template <typename T, bool INV>
struct Dft<T, 2, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[2]) { Bfly<T, 2, INV>::run(v); }
};
template <typename T, bool INV>
struct Dft<T, 3, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[3]) { Bfly<T, 3, INV>::run(v); }
};
template <typename T, bool INV>
struct Dft<T, 4, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[4]) { Bfly<T, 4, INV>::run(v); }
};
template <typename T, bool INV>
struct Dft<T, 5, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[5]) { Bfly<T, 5, INV>::run(v); }
};
template <typename T, bool INV>
struct Dft<T, 8, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[8]) { Bfly<T, 8, INV>::run(v); }
};

// multiply by exp(s*2 pi i e/m), s = -1 forward, given cos/sin of 2 pi e/m
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> twc(cplx<T> a, T c, T s)
{
    const T sn = INV ? s : -s;
    return {a.x * c - a.y * sn, a.x * sn + a.y * c};
}

// 6 = 2 x 3: j = a + 2b, X[kb + 3 ka]
template <typename T, bool INV>
struct Dft<T, 6, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[6])
    {
        const T  h = (T)0.5, r3 = (T)0.86602540378443864676;
        cplx<T> e[3] = {v[0], v[2], v[4]}, o[3] = {v[1], v[3], v[5]};
        Bfly<T, 3, INV>::run(e);
        Bfly<T, 3, INV>::run(o);
        o[1] = twc<T, INV>(o[1], h, r3);  // W6^1
        o[2] = twc<T, INV>(o[2], -h, r3); // W6^2
#pragma unroll
        for (int kb = 0; kb < 3; ++kb) {
            v[kb]     = cadd(e[kb], o[kb]);
            v[kb + 3] = csub(e[kb], o[kb]);
        }
    }
};

// 16 = 4 x 4: j = a + 4b; U[a][kb] = DFT4_b x[a+4b]; U *= W16^(a kb); X[kb + 4 ka] = DFT4_a U
template <typename T, bool INV>
struct Dft<T, 16, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[16])
    {
        const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
        const T h  = (T)0.70710678118654752440;
        cplx<T> u[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            cplx<T> t[4] = {v[a], v[a + 4], v[a + 8], v[a + 12]};
            Bfly<T, 4, INV>::run(t);
#pragma unroll
            for (int kb = 0; kb < 4; ++kb)
                u[a][kb] = t[kb];
        }
        // twiddles W16^(a kb): (1,1)=1 (1,2)=2 (1,3)=3 (2,1)=2 (2,2)=4 (2,3)=6 (3,1)=3 (3,2)=6 (3,3)=9
        u[1][1] = twc<T, INV>(u[1][1], c1, s1);
        u[1][2] = twc<T, INV>(u[1][2], h, h);
        u[1][3] = twc<T, INV>(u[1][3], s1, c1);
        u[2][1] = twc<T, INV>(u[2][1], h, h);
        u[2][2] = rot90<T, INV>(u[2][2]);
        u[2][3] = twc<T, INV>(u[2][3], -h, h);
        u[3][1] = twc<T, INV>(u[3][1], s1, c1);
        u[3][2] = twc<T, INV>(u[3][2], -h, h);
        u[3][3] = twc<T, INV>(u[3][3], -c1, -s1);
#pragma unroll
        for (int kb = 0; kb < 4; ++kb) {
            cplx<T> t[4] = {u[0][kb], u[1][kb], u[2][kb], u[3][kb]};
            Bfly<T, 4, INV>::run(t);
#pragma unroll
            for (int ka = 0; ka < 4; ++ka)
                v[kb + 4 * ka] = t[ka];
        }
    }
};

// Phase 1 of the line FFT: DFT of size N2 over the worker's values, then the
// twiddle W_n^(w*k2) from the n-entry table (forward roots; conjugated when INV).
template <typename T, int N1, int N2, bool INV>
__device__ __forceinline__ void line_phase1(cplx<T> (&v)[N2], int w, const cplx<T> *__restrict__ tw)
{
    Dft<T, N2, INV>::run(v);
#pragma unroll
    for (int k2 = 1; k2 < N2; ++k2) {
        cplx<T> t = tw[w * k2];
        if (INV)
            t.y = -t.y;
        v[k2] = cmul(v[k2], t);
    }
}

// sizes with a register plan: n -> (N1, N2), N1 >= N2
__host__ __device__ constexpr int reg_n1(int n)
{
    return n == 256 ? 16 : n == 128 ? 16 : n == 96 ? 16 : n == 80 ? 16 : n == 64 ? 8 : n == 48 ? 8 : n == 40 ? 8
         : n == 32 ? 8 : n == 24 ? 8 : n == 16 ? 4 : 0;
}

} // namespace fansgpu
