"""Host checks of two identities the GPU path relies on (numpy only, no GPU).

* The FP32 convolution takes <r, s> from the spectra (Parseval): for real r and
  s = sign * c2r(G . r2c(r)) (unnormalised transforms, G holding 1/N), <r, s> =
  sign * sum over the half spectrum of w(kz) Re(r^ conj(G r^)) with w = 1 at kz = 0
  and kz = nz/2 and 2 in between.
* The Green's table kernel evaluates the weighted contraction of solver.h:177-186,
  block_ij = sum_pq K0_ij[p][q] Re(A_p conj A_q), as sums over the 14 classes of
  node offsets d = x_p - x_q (d and -d together) times cos(theta . d).
"""
import numpy as np


def _half_weights(nz):
    w = np.full(nz // 2 + 1, 2.0)
    w[0] = 1.0
    w[-1] = 1.0  # nz even: kz = nz/2
    return w


def test_parseval_half_spectrum_dot():
    rng = np.random.default_rng(5)
    nx, ny, nz, C = 6, 10, 8, 3
    N = nx * ny * nz
    r = rng.standard_normal((C, nx, ny, nz))
    # a Green's-like operator of a real field: real symmetric per frequency and even in k
    M = rng.standard_normal((C, C))
    M = 0.5 * (M + M.T)
    cx = np.cos(2 * np.pi * np.arange(nx) / nx)[:, None, None]
    cy = np.cos(2 * np.pi * np.arange(ny) / ny)[None, :, None]
    cz = np.cos(2 * np.pi * np.arange(nz // 2 + 1) / nz)[None, None, :]
    G = M[:, :, None, None, None] * (1.5 + cx + 0.5 * cy + 0.25 * cz) / N
    rh = np.fft.rfftn(r, axes=(1, 2, 3))
    yh = np.einsum("abxyz,bxyz->axyz", G, rh)
    sign = -1.0
    s = sign * np.fft.irfftn(yh, s=(nx, ny, nz), axes=(1, 2, 3)) * N  # unnormalised c2r
    direct = float(np.sum(r * s))
    w = _half_weights(nz)
    spectral = sign * float(np.sum(w * np.real(rh * np.conj(yh))))
    assert abs(direct - spectral) <= 1e-12 * max(abs(direct), 1.0)


def _offset_class(d):
    d = list(d)
    for v in d:
        if v != 0:
            if v < 0:
                d = [-u for u in d]
            break
    return tuple(d)


def test_green_block_by_offset_classes():
    rng = np.random.default_rng(6)
    C = 3
    NC = 8 * C
    K0 = rng.standard_normal((NC, NC))
    K0 = 0.5 * (K0 + K0.T)  # the reference element stiffness is symmetric
    nodes = [(p & 1, (p >> 1) & 1, p >> 2) for p in range(8)]
    classes = sorted({_offset_class(tuple(a - b for a, b in zip(nodes[p], nodes[q])))
                      for p in range(8) for q in range(8)})
    assert len(classes) == 14
    for _ in range(20):
        th = rng.uniform(-np.pi, np.pi, 3)
        A = np.array([np.exp(1j * np.dot(th, x)) for x in nodes])
        for i in range(C):
            for j in range(C):
                blk = K0[8 * i:8 * i + 8, 8 * j:8 * j + 8]
                pairs = sum(blk[p, q] * np.real(A[p] * np.conj(A[q])) for p in range(8) for q in range(8))
                T = {c: 0.0 for c in classes}
                for p in range(8):
                    for q in range(8):
                        T[_offset_class(tuple(a - b for a, b in zip(nodes[p], nodes[q])))] += blk[p, q]
                by_class = sum(T[c] * np.cos(np.dot(th, c)) for c in classes)
                assert abs(pairs - by_class) <= 1e-12 * max(1.0, np.abs(blk).sum())
