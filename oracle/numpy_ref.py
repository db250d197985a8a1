"""Independent numpy restatement of the FANS solve path (small grids only).

TEST INFRASTRUCTURE ONLY: used to cross-check the C oracle (fans_oracle.c)
with a different FFT (numpy.fft / pocketfft), a different pseudo-inverse
(LAPACK eigh) and a vectorised stencil.  Citations are to FANS v0.6.2.
"""
from __future__ import annotations

import numpy as np

SQRT_HALF = 7.071067811865476e-01


def basic_B(x, y, z, le):
    """Matmodel::Compute_basic_B (matmodel.h:158-188)."""
    lx, ly, lz = le
    w = lambda t, b: t if b else 1.0 - t  # noqa: E731
    dw = lambda b: 1.0 if b else -1.0  # noqa: E731
    out = np.zeros((3, 8))
    for p in range(8):
        bx, by, bz = p & 1, (p >> 1) & 1, (p >> 2) & 1
        out[0, p] = dw(bx) * w(y, by) * w(z, bz) / lx
        out[1, p] = w(x, bx) * dw(by) * w(z, bz) / ly
        out[2, p] = w(x, bx) * w(y, by) * dw(bz) / lz
    return out


def model_B(c, x, y, z, le):
    b = basic_B(x, y, z, le)
    if c == 1:
        return b
    out = np.zeros((6, 24))
    for q in range(8):
        out[0, 3 * q + 0] = b[0, q]
        out[1, 3 * q + 1] = b[1, q]
        out[2, 3 * q + 2] = b[2, q]
        out[3, 3 * q + 0] = SQRT_HALF * b[1, q]
        out[3, 3 * q + 1] = SQRT_HALF * b[0, q]
        out[4, 3 * q + 0] = SQRT_HALF * b[2, q]
        out[4, 3 * q + 2] = SQRT_HALF * b[0, q]
        out[5, 3 * q + 1] = SQRT_HALF * b[2, q]
        out[5, 3 * q + 2] = SQRT_HALF * b[1, q]
    return out


def gauss_B(c, fe, le):
    """Construct_B (matmodel.h:104-155); returns (ngp, nstr, 8c)."""
    if fe == "HEX8R":
        return model_B(c, 0.5, 0.5, 0.5, le)[None]
    m, p = 0.5 - np.sqrt(3.0) / 6.0, 0.5 + np.sqrt(3.0) / 6.0
    pts = [(m, m, m), (p, m, m), (m, p, m), (p, p, m), (m, m, p), (p, m, p), (m, p, p), (p, p, p)]
    Bs = np.array([model_B(c, *pt, le) for pt in pts])
    if fe == "BBAR" and c == 3:
        Bv = model_B(c, 0.5, 0.5, 0.5, le)
        vol_bar = Bv[:3].sum(0) / 3.0
        for g in range(8):
            vol_full = Bs[g, :3].sum(0) / 3.0
            Bs[g, :3] = Bs[g, :3] - vol_full + vol_bar
    return Bs


def element_stiffness(Bs, C, ve):
    return sum(B.T @ C @ B for B in Bs) * ve / len(Bs)


def node_shift(f, p):
    """f at node idx[p] of every element (element (x,y,z) <- node offset bits of p)."""
    return np.roll(f, shift=(-(p & 1), -((p >> 1) & 1), -((p >> 2) & 1)), axis=(0, 1, 2))


def gather_elements(u):
    """u [x,y,z,c] -> ue [x,y,z, 8*c] node-major (iterateCubes order, solver.h:318-385)."""
    return np.concatenate([node_shift(u, p) for p in range(8)], axis=-1)


def scatter_elements(re, c):
    """re [x,y,z,8c] -> r [x,y,z,c] (scatter-add to the element's 8 nodes)."""
    r = np.zeros(re.shape[:3] + (c,))
    for p in range(8):
        r += np.roll(re[..., c * p:c * (p + 1)], shift=(p & 1, (p >> 1) & 1, (p >> 2) & 1), axis=(0, 1, 2))
    return r


def apply_linear(ms, Kph, d):
    c = d.shape[-1]
    ue = gather_elements(d)
    ue = ue - np.tile(d, (1, 1, 1, 8))
    re = np.einsum("xyzij,xyzj->xyzi", Kph[ms], ue)
    return scatter_elements(re, c)


def linear_residual(ms, Bs, Cph, ve, g0, u):
    """compute_residual for linear laws: r_e = sum_gp B^T C (B ue + g0) ve/ngp."""
    c = u.shape[-1]
    ue = gather_elements(u) - np.tile(u, (1, 1, 1, 8))
    C = Cph[ms]
    re = 0.0
    for B in Bs:
        eps = np.einsum("ij,xyzj->xyzi", B, ue) + g0
        sig = np.einsum("xyzij,xyzj->xyzi", C, eps)
        re = re + np.einsum("ji,xyzj->xyzi", B, sig)
    return scatter_elements(re * ve / len(Bs), c)


def green(n, c, K0n):
    """computeFundamentalSolution (solver.h:145-204) with numpy; returns G[kx,ky,kz,c,c]."""
    nx, ny, nz = n
    nzh = nz // 2 + 1
    K0 = np.zeros_like(K0n)
    ncol = 8 * c
    for i in range(ncol):
        for j in range(ncol):
            K0[(i % c) * 8 + i // c, (j % c) * 8 + j // c] = K0n[i, j]
    ex = np.exp(2j * np.pi * np.arange(nx) / nx)
    ey = np.exp(2j * np.pi * np.arange(ny) / ny)
    ez = np.exp(2j * np.pi * np.arange(nzh) / nz)
    EX, EY, EZ = np.meshgrid(ex, ey, ez, indexing="ij")
    one = np.ones_like(EX)
    A = np.stack([one, EX, EY, EX * EY, EZ, EX * EZ, EZ * EY, EX * EY * EZ], axis=-1)
    AA = np.einsum("...p,...q->...pq", A.real, A.real) + np.einsum("...p,...q->...pq", A.imag, A.imag)
    blk = np.zeros((nx, ny, nzh, c, c))
    for i in range(c):
        for j in range(c):
            blk[..., i, j] = np.einsum("pq,...pq->...", K0[8 * i:8 * i + 8, 8 * j:8 * j + 8], AA)
    w, V = np.linalg.eigh(blk)
    winv = np.where(np.abs(w) > 1e-14, 1.0 / np.where(w == 0, 1.0, w), 0.0)
    G = np.einsum("...ik,...k,...jk->...ij", V, winv, V)
    G[0, 0, 0] = 0.0
    return G / (nx * ny * nz)


def convolve(G, r):
    nz = r.shape[2]
    rh = np.fft.rfftn(r, axes=(0, 1, 2))
    sh = np.einsum("...ij,...j->...i", G, rh)
    return np.fft.irfftn(sh, s=r.shape[:3], axes=(0, 1, 2)) * r.shape[0] * r.shape[1] * nz


def cg_linear(ms, Bs, Cph, Kph, ve, G, g0, u, tol, n_it, measure="L2", typ="relative"):
    """SolverCG::internalSolve, linear branch (solverCG.h:62-117)."""

    def norm(r):
        a = np.abs(r)
        return {"L1": a.sum(), "L2": np.sqrt((a * a).sum()), "Linfinity": a.max()}[measure]

    r = linear_residual(ms, Bs, Cph, ve, g0, u)
    s = np.zeros_like(u)
    d = np.zeros_like(u)
    err_all = [norm(r)]
    it = 0
    err = 100.0 if typ == "relative" else err_all[0]
    delta = 1.0
    while it < n_it and err > tol:
        deltamid = (r * s).sum()
        s = -convolve(G, r)
        delta0, delta = delta, (r * s).sum()
        d = s + max(0.0, (delta - deltamid) / delta0) * d
        rnew = apply_linear(ms, Kph, d)
        alpha = delta / (d * rnew).sum()
        r = r - alpha * rnew
        u = u - alpha * d
        it += 1
        err_all.append(norm(r))
        err = err_all[-1] / err_all[0] if typ == "relative" else err_all[-1]
    return u, r, it, np.array(err_all)


def strain_stress_avg(ms, Bs, Cph, g0, u):
    ue = gather_elements(u)
    C = Cph[ms]
    se, ss = 0.0, 0.0
    for B in Bs:
        eps = np.einsum("ij,xyzj->xyzi", B, ue) + g0
        se = se + eps
        ss = ss + np.einsum("xyzij,xyzj->xyzi", C, eps)
    se, ss = se / len(Bs), ss / len(Bs)
    return se.reshape(-1, se.shape[-1]).mean(0), ss.reshape(-1, ss.shape[-1]).mean(0)
