"""Seeded synthetic microstructures standing in for the reference's HDF5 inputs.

`spheres` builds a periodic two-phase box (uint8 phase ids: 0 matrix, 1
inclusion) of non-overlapping spheres by random sequential addition: centres
uniform in [0, n)^3 from numpy's PCG64 `default_rng(seed)`, accepted when the
periodic minimum-image distance to every accepted centre is >= 2r, stopping at
round(vf n^3 / (4/3 pi r^3)) spheres (optionally capped) or 10^6 attempts.  A
voxel (i,j,k) is inclusion when its centre (i+1/2, j+1/2, k+1/2) lies within r
of a centre (periodic).
"""
from __future__ import annotations

import math

import numpy as np


def spheres(n, radius, vf, seed, max_spheres=None, max_attempts=1_000_000):
    n = int(n)
    target = int(round(vf * n ** 3 / (4.0 / 3.0 * math.pi * radius ** 3)))
    if max_spheres is not None:
        target = min(target, int(max_spheres))
    rng = np.random.default_rng(seed)
    cell = 2.0 * radius
    ncell = max(1, int(n // cell))
    csize = n / ncell
    grid: dict = {}
    centres = []
    attempts = 0
    min_d2 = (2.0 * radius) ** 2
    batch = 4096
    while len(centres) < target and attempts < max_attempts:
        cand = rng.uniform(0.0, n, size=(batch, 3))
        for c in cand:
            attempts += 1
            if attempts > max_attempts:
                break
            ci = (int(c[0] // csize) % ncell, int(c[1] // csize) % ncell, int(c[2] // csize) % ncell)
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        key = ((ci[0] + dx) % ncell, (ci[1] + dy) % ncell, (ci[2] + dz) % ncell)
                        for o in grid.get(key, ()):
                            d = np.abs(c - o)
                            d = np.minimum(d, n - d)
                            if d @ d < min_d2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                centres.append(c)
                grid.setdefault(ci, []).append(c)
                if len(centres) >= target:
                    break
    ms = np.zeros((n, n, n), dtype=np.uint8)
    R = int(math.ceil(radius)) + 1
    off = np.arange(-R, R + 1)
    for c in centres:
        base = np.floor(c).astype(int)
        ix = (base[0] + off) % n
        iy = (base[1] + off) % n
        iz = (base[2] + off) % n
        px = base[0] + off + 0.5 - c[0]
        py = base[1] + off + 0.5 - c[1]
        pz = base[2] + off + 0.5 - c[2]
        d2 = px[:, None, None] ** 2 + py[None, :, None] ** 2 + pz[None, None, :] ** 2
        mask = d2 <= radius * radius
        sub = ms[np.ix_(ix, iy, iz)]
        sub[mask] = 1
        ms[np.ix_(ix, iy, iz)] = sub
    return ms, np.array(centres)


def laminate(n, axis=0, frac=0.5):
    """Two-layer periodic laminate along `axis` (known-answer microstructure)."""
    ms = np.zeros((n, n, n) if np.isscalar(n) else tuple(n), dtype=np.uint8)
    m = ms.shape[axis]
    sl = [slice(None)] * 3
    sl[axis] = slice(int(round(m * frac)), m)
    ms[tuple(sl)] = 1
    return ms


BATCH_EDGES = (32, 48, 64, 80, 96)


def batch_workload(count=64, seed_base=100):
    """The batched-micro-problem workload: instance k uses seed seed_base + k for
    its edge (uniform over BATCH_EDGES) and its spheres; even k is thermal
    (r = 4, vf 0.20, conductivities 1 and 10, three unit gradients), odd k
    elastic (r = 6, vf 0.30, six unit strains).  The sphere count follows the
    volume fraction; random sequential addition stops at its attempt cap when a
    small box cannot hold them all."""
    out = []
    for k in range(count):
        rng = np.random.default_rng(seed_base + k)
        n = int(BATCH_EDGES[int(rng.integers(0, len(BATCH_EDGES)))])
        thermal = k % 2 == 0
        ms, centres = spheres(n, 4 if thermal else 6, 0.20 if thermal else 0.30, seed_base + k,
                              max_attempts=200_000)
        out.append({"k": k, "n": n, "thermal": thermal, "ms": ms, "spheres": len(centres)})
    return out
