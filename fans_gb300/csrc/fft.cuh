// fft.cuh -- shared-memory mixed-radix Stockham FFT used by the convolution passes.
//
// A CTA transforms a batch of lines held in shared memory.  Element i of line L
// lives at  base(L) + i*es  with  base(L) = (L / lpg) * gs + (L % lpg),  which
// covers the three pass layouts:
//   z pass: lines are rows,               lpg = 1,  gs = row stride, es = 1
//   y pass: lines are kz columns of a tile, lpg = KC, gs = 0,          es = KC
//   x pass: (component, kz column) lines,  lpg = KC, gs = n*KC,        es = KC
// Each stage reads buffer A and writes buffer B (ping-pong), so a thread can
// process any number of butterflies without holding them across a barrier.
// Twiddles: tw[q] = exp(-2 pi i q / n), q < n (forward roots; the inverse uses
// their conjugates).  Forward = FFTW_FORWARD sign, both directions unnormalised.
#pragma once
#include "fans_common.cuh"

namespace fansgpu {

constexpr int kMaxRadices = 16;

struct FftDim {
    int n;
    int nrad;
    int rad[kMaxRadices];
};

// v[o] = sum_r v[r] * exp(s * 2 pi i r o / R), s = -1 forward, +1 inverse.
template <typename T, int R, bool INV>
struct Bfly;

template <typename T, bool INV>
struct Bfly<T, 2, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[2])
    {
        cplx<T> a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

// multiply by -i (forward) or +i (inverse)
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> rot90(cplx<T> a)
{
    return INV ? cplx<T>{-a.y, a.x} : cplx<T>{a.y, -a.x};
}

template <typename T, bool INV>
struct Bfly<T, 4, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[4])
    {
        cplx<T> t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        cplx<T> t2 = cadd(v[1], v[3]), t3 = rot90<T, INV>(csub(v[1], v[3]));
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    }
};

template <typename T, bool INV>
struct Bfly<T, 8, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[8])
    {
        const T h = (T)0.70710678118654752440;
        cplx<T> e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
        Bfly<T, 4, INV>::run(e);
        Bfly<T, 4, INV>::run(o);
        // twiddles exp(s*2 pi i k/8), k = 0..3
        cplx<T> o1 = o[1], o3 = o[3];
        if (!INV) {
            o[1] = {h * (o1.x + o1.y), h * (o1.y - o1.x)};   // * (h - i h)
            o[3] = {h * (-o3.x + o3.y), h * (-o3.y - o3.x)}; // * (-h - i h)
        } else {
            o[1] = {h * (o1.x - o1.y), h * (o1.y + o1.x)};   // * (h + i h)
            o[3] = {h * (-o3.x - o3.y), h * (-o3.y + o3.x)}; // * (-h + i h)
        }
        o[2] = rot90<T, INV>(o[2]);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k]     = cadd(e[k], o[k]);
            v[k + 4] = csub(e[k], o[k]);
        }
    }
};

template <typename T, bool INV>
struct Bfly<T, 3, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[3])
    {
        const T c = (T)0.86602540378443864676; // sqrt(3)/2
        cplx<T> a = v[0], t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
        cplx<T> m = {a.x - (T)0.5 * t.x, a.y - (T)0.5 * t.y};
        // s*i*c*u with s = -1 forward
        cplx<T> w = INV ? cplx<T>{-c * u.y, c * u.x} : cplx<T>{c * u.y, -c * u.x};
        v[0] = cadd(a, t);
        v[1] = cadd(m, w);
        v[2] = csub(m, w);
    }
};

template <typename T, bool INV>
struct Bfly<T, 5, INV> {
    __device__ __forceinline__ static void run(cplx<T> (&v)[5])
    {
        const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
        const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
        cplx<T> a = v[0];
        cplx<T> t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        cplx<T> t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
        cplx<T> m1 = {a.x + c1 * t1.x + c2 * t2.x, a.y + c1 * t1.y + c2 * t2.y};
        cplx<T> m2 = {a.x + c2 * t1.x + c1 * t2.x, a.y + c2 * t1.y + c1 * t2.y};
        cplx<T> p1 = {s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y};
        cplx<T> p2 = {s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y};
        // s*i*p
        cplx<T> q1 = INV ? cplx<T>{-p1.y, p1.x} : cplx<T>{p1.y, -p1.x};
        cplx<T> q2 = INV ? cplx<T>{-p2.y, p2.x} : cplx<T>{p2.y, -p2.x};
        v[0] = cadd(a, cadd(t1, t2));
        v[1] = cadd(m1, q1);
        v[4] = csub(m1, q1);
        v[2] = cadd(m2, q2);
        v[3] = csub(m2, q2);
    }
};

__device__ __forceinline__ int line_base(int L, int lpg, int gs)
{
    return (L / lpg) * gs + (L % lpg);
}

// One Stockham stage of compile-time radix R.
template <typename T, int R, bool INV, bool LINE_FAST>
__device__ __forceinline__ void fft_stage(const cplx<T> *__restrict__ src, cplx<T> *__restrict__ dst, int n, int Ns,
                                          int nl, int lpg, int gs, int es, const cplx<T> *__restrict__ tw, int tid,
                                          int nthr)
{
    const int m = n / R, tmul = n / (Ns * R), total = m * nl;
    for (int w = tid; w < total; w += nthr) {
        int L, j;
        if (LINE_FAST) {
            L = w % nl;
            j = w / nl;
        } else {
            j = w % m;
            L = w / m;
        }
        const int base = line_base(L, lpg, gs);
        const int k    = j % Ns;
        cplx<T>   v[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
            v[r] = src[base + (j + r * m) * es];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                cplx<T> t = tw[r * k * tmul];
                if (INV)
                    t.y = -t.y;
                v[r] = cmul(v[r], t);
            }
        }
        Bfly<T, R, INV>::run(v);
        const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r)
            dst[base + (idxD + r * Ns) * es] = v[r];
    }
}

// Radix R > 8 or 7: naive DFT per butterfly (rarely used sizes).
template <typename T, bool INV, bool LINE_FAST>
__device__ void fft_stage_generic(const cplx<T> *__restrict__ src, cplx<T> *__restrict__ dst, int R, int n, int Ns,
                                  int nl, int lpg, int gs, int es, const cplx<T> *__restrict__ tw, int tid, int nthr)
{
    const int m = n / R, tmul = n / (Ns * R), total = m * nl, rstep = n / R;
    for (int w = tid; w < total; w += nthr) {
        int L, j;
        if (LINE_FAST) {
            L = w % nl;
            j = w / nl;
        } else {
            j = w % m;
            L = w / m;
        }
        const int base = line_base(L, lpg, gs);
        const int k    = j % Ns;
        const int idxD = (j / Ns) * Ns * R + k;
        for (int o = 0; o < R; ++o) {
            cplx<T> acc = {0, 0};
            for (int r = 0; r < R; ++r) {
                cplx<T> x = src[base + (j + r * m) * es];
                int     q = (r * k * tmul + ((r * o) % R) * rstep) % n;
                cplx<T> t = tw[q];
                if (INV)
                    t.y = -t.y;
                acc = cadd(acc, cmul(x, t));
            }
            dst[base + (idxD + o * Ns) * es] = acc;
        }
    }
}

// Full transform of nl lines; returns the buffer that holds the result (a or b).
template <typename T, bool INV, bool LINE_FAST>
__device__ cplx<T> *fft_lines(cplx<T> *a, cplx<T> *b, const FftDim &d, int nl, int lpg, int gs, int es,
                              const cplx<T> *tw, int tid, int nthr)
{
    int Ns = 1;
    for (int s = 0; s < d.nrad; ++s) {
        const int R = d.rad[s];
        switch (R) {
        case 2: fft_stage<T, 2, INV, LINE_FAST>(a, b, d.n, Ns, nl, lpg, gs, es, tw, tid, nthr); break;
        case 3: fft_stage<T, 3, INV, LINE_FAST>(a, b, d.n, Ns, nl, lpg, gs, es, tw, tid, nthr); break;
        case 4: fft_stage<T, 4, INV, LINE_FAST>(a, b, d.n, Ns, nl, lpg, gs, es, tw, tid, nthr); break;
        case 5: fft_stage<T, 5, INV, LINE_FAST>(a, b, d.n, Ns, nl, lpg, gs, es, tw, tid, nthr); break;
        case 8: fft_stage<T, 8, INV, LINE_FAST>(a, b, d.n, Ns, nl, lpg, gs, es, tw, tid, nthr); break;
        default: fft_stage_generic<T, INV, LINE_FAST>(a, b, R, d.n, Ns, nl, lpg, gs, es, tw, tid, nthr); break;
        }
        __syncthreads();
        cplx<T> *t = a;
        a          = b;
        b          = t;
        Ns *= R;
    }
    return a;
}

} // namespace fansgpu
