"""Seeded synthetic meshes with the shapes of the LSCM benchmark workloads.

No public dataset is involved; every input is procedural and deterministic (numpy PCG64
with a fixed seed).  Positions are generated in float32 and promoted to float64, as the
workloads specify ("f32 positions, f64 assembly").

* :func:`height_field` — an n x n vertex grid on [0,1]^2 lifted to
  z = amp * sum_k a_k sin(2 pi (f_k . (x, y)) + phi_k), a_k ~ U(0.2, 1), integer frequency
  vectors with entries in [1, 6], phi_k ~ U(0, 2 pi): one open chart.
  (1024^2 / 8 sines / 0.15 and 2048^2 / 16 sines / 0.3.)
* :func:`disks` — n_charts independent disk patches, triangle counts log-uniform in
  [t_min, t_max]: a Delaunay-style polar grid (ring k has 6k vertices, zipper-triangulated
  between rings, 6 R^2 triangles for R rings) of radius 1; each interior vertex is displaced
  radially by 0.1 * N(0,1) of the ring spacing and along the normal by 0.1 * N(0,1) of the
  ring spacing, both noise fields smoothed by 3 Laplacian (neighbour-average) steps.  The
  boundary ring stays on the unit circle.  One chart per disk.
* :func:`sh_sphere` — an n_lat x n_lon latitude-longitude sphere, radius
  1 + amp * sum of n_sh seeded random-phase real spherical harmonics of degree <= 6, cut at
  one meridian (no wrap-around between the last and first longitude) and at both poles (the
  latitudes stop half a step short of each pole): one disk chart whose border is the cut.
  (512 x 1024, 8 harmonics, 0.05: the differentiation workload.)
"""
from __future__ import annotations

import numpy as np


def grid_faces(nx: int, ny: int) -> np.ndarray:
    """Faces of an nx x ny vertex grid (row-major), two triangles per quad, in the
    reference's grid winding (unwrap/src/meshgen.rs:143-153)."""
    j, i = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    a = (j * nx + i).ravel()
    b = a + 1
    c = a + nx
    d = c + 1
    f = np.empty((a.size * 2, 3), np.int32)
    f[0::2] = np.stack([a, b, d], 1)
    f[1::2] = np.stack([a, d, c], 1)
    return f


def height_field(n: int = 1024, n_sines: int = 8, amp: float = 0.15, seed: int = 2):
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.uniform(0.2, 1.0, n_sines)
    fr = rng.integers(1, 7, size=(n_sines, 2))
    ph = rng.uniform(0.0, 2.0 * np.pi, n_sines)
    t = np.linspace(0.0, 1.0, n)
    y, x = np.meshgrid(t, t, indexing="ij")
    z = np.zeros_like(x)
    for k in range(n_sines):
        z += a[k] * np.sin(2.0 * np.pi * (fr[k, 0] * x + fr[k, 1] * y) + ph[k])
    z *= amp
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32).astype(np.float64)
    return pos, grid_faces(n, n)


def _polar_disk(R: int):
    """Vertices (ring, angle) and faces of a polar disk with R rings (6 R^2 triangles)."""
    ring_start = [0]
    counts = [1] + [6 * k for k in range(1, R + 1)]
    for c in counts:
        ring_start.append(ring_start[-1] + c)
    nv = ring_start[-1]
    rad = np.zeros(nv)
    ang = np.zeros(nv)
    ring = np.zeros(nv, np.int64)
    for k in range(1, R + 1):
        s, m = ring_start[k], counts[k]
        off = 0.5 * (k % 2)
        ang[s:s + m] = 2.0 * np.pi * (np.arange(m) + off) / m
        rad[s:s + m] = k / R
        ring[s:s + m] = k
    faces = []
    # ring 0 -> 1: fan
    for i in range(6):
        faces.append((0, 1 + i, 1 + (i + 1) % 6))
    for k in range(2, R + 1):
        si, mi = ring_start[k - 1], counts[k - 1]
        so, mo = ring_start[k], counts[k]
        ai = ang[si:si + mi]
        ao = ang[so:so + mo]
        # zipper: advance the ring whose next vertex comes first in angle
        i = j = 0
        while i < mi or j < mo:
            ni = ai[(i + 1) % mi] + (2 * np.pi if i + 1 >= mi else 0.0)
            no = ao[(j + 1) % mo] + (2 * np.pi if j + 1 >= mo else 0.0)
            if j < mo and (i >= mi or no <= ni):
                faces.append((si + i % mi, so + j % mo, so + (j + 1) % mo))
                j += 1
            else:
                faces.append((si + i % mi, so + j % mo, si + (i + 1) % mi))
                i += 1
    return rad, ang, ring, np.asarray(faces, np.int32)


def _smooth(vals, faces, nv, steps=3):
    """Neighbour-average (Laplacian) smoothing over the triangle graph."""
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    e = np.concatenate([e, e[:, ::-1]])
    deg = np.bincount(e[:, 0], minlength=nv).astype(np.float64)
    for _ in range(steps):
        acc = np.bincount(e[:, 0], weights=vals[e[:, 1]], minlength=nv)
        vals = 0.5 * vals + 0.5 * acc / np.maximum(deg, 1.0)
    return vals


_DISK_CACHE: dict = {}


def disks(n_charts: int = 4096, t_min: int = 50, t_max: int = 50_000, seed: int = 3):
    """Packed patches: (vert_off, tri_off, p3 (V, 3) f64, tris (T, 3) i32 patch-local)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.exp(rng.uniform(np.log(t_min), np.log(t_max), n_charts))
    Rs = np.maximum(1, np.rint(np.sqrt(t / 6.0)).astype(np.int64))
    vert_off = [0]
    tri_off = [0]
    P, F = [], []
    for R in Rs:
        R = int(R)
        if R not in _DISK_CACHE:
            _DISK_CACHE[R] = _polar_disk(R)
        rad, ang, ring, faces = _DISK_CACHE[R]
        nv = rad.size
        interior = ring < R
        h = 1.0 / R
        nr = _smooth(rng.standard_normal(nv), faces, nv) * 0.1 * h
        nz = _smooth(rng.standard_normal(nv), faces, nv) * 0.1 * h
        r = rad + np.where(interior & (ring > 0), nr, 0.0)
        z = np.where(interior, nz, 0.0)
        p = np.stack([r * np.cos(ang), r * np.sin(ang), z], 1).astype(np.float32).astype(np.float64)
        P.append(p)
        F.append(faces)
        vert_off.append(vert_off[-1] + nv)
        tri_off.append(tri_off[-1] + len(faces))
    return (np.asarray(vert_off, np.int64), np.asarray(tri_off, np.int64), np.concatenate(P),
            np.concatenate(F).astype(np.int32))


def _assoc_legendre(l: int, m: int, x: np.ndarray) -> np.ndarray:
    """P_l^m(x) for 0 <= m <= l by the standard upward recurrence in l (no Condon-Shortley
    phase)."""
    pmm = np.ones_like(x)
    if m > 0:
        s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
        f = 1.0
        for _ in range(m):
            pmm = pmm * f * s
            f += 2.0
    if l == m:
        return pmm
    pm1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pm1
    for ll in range(m + 2, l + 1):
        pll = ((2 * ll - 1) * x * pm1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pm1 = pm1, pll
    return pm1


def sh_sphere(n_lat: int = 512, n_lon: int = 1024, n_sh: int = 8, amp: float = 0.05, seed: int = 4):
    """Returns (positions (n_lat * n_lon, 3), faces): rows are latitudes from north to south,
    theta_r = pi (r + 1/2) / n_lat, columns longitudes phi_c = 2 pi c / n_lon.  Each harmonic:
    degree l ~ U{1..6}, order m ~ U{0..l}, phase ~ U(0, 2 pi), orthonormal scaling
    sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!) (times sqrt 2 for m > 0)."""
    from math import factorial, pi, sqrt

    rng = np.random.Generator(np.random.PCG64(seed))
    ls = rng.integers(1, 7, n_sh)
    ms = np.array([rng.integers(0, l + 1) for l in ls])
    ph = rng.uniform(0.0, 2.0 * np.pi, n_sh)
    theta = np.pi * (np.arange(n_lat) + 0.5) / n_lat
    phi = 2.0 * np.pi * np.arange(n_lon) / n_lon
    T, Ph = np.meshgrid(theta, phi, indexing="ij")
    ct = np.cos(T)
    r = np.ones_like(T)
    for k in range(n_sh):
        l, m = int(ls[k]), int(ms[k])
        norm = sqrt((2 * l + 1) / (4 * pi) * factorial(l - m) / factorial(l + m)) * (sqrt(2.0) if m > 0 else 1.0)
        r += amp * norm * _assoc_legendre(l, m, ct) * np.cos(m * Ph + ph[k])
    st = np.sin(T)
    pos = np.stack([(r * st * np.cos(Ph)).ravel(), (r * st * np.sin(Ph)).ravel(), (r * ct).ravel()], 1)
    return pos.astype(np.float32).astype(np.float64), grid_faces(n_lon, n_lat)


def disk_unknowns(vert_off, tri_off, tris) -> int:
    """Unknowns (2 x free vertices) of a batch of open disk patches, from topology alone: the
    reference pins every vertex of a border loop (unwrap/src/lscm.rs:524-529), and a disk's
    border loop is the set of vertices on an edge that only one triangle uses."""
    vo = np.asarray(vert_off, np.int64)
    to = np.asarray(tri_off, np.int64)
    t = np.asarray(tris, np.int64).reshape(-1, 3)
    # global vertex ids (patch-local + the patch's first vertex)
    base = np.repeat(vo[:-1], np.diff(to))
    g = t + base[:, None]
    e = np.concatenate([g[:, [0, 1]], g[:, [1, 2]], g[:, [2, 0]]])
    e.sort(axis=1)
    key = e[:, 0] * (int(vo[-1]) + 1) + e[:, 1]
    uniq, cnt = np.unique(key, return_counts=True)
    border = uniq[cnt == 1]
    on_border = np.zeros(int(vo[-1]), bool)
    on_border[border // (int(vo[-1]) + 1)] = True
    on_border[border % (int(vo[-1]) + 1)] = True
    return int(2 * (int(vo[-1]) - int(on_border.sum())))

