"""Seeded synthetic triangle meshes for the OptCuts inner loop.

The reference's own benchmark meshes (input/benchmark/*.obj, at most 20k
triangles) stop well short of the sizes this library targets, so the
workloads are generated here with numpy from fixed seeds:

* ``icosphere(level, noise, seed)``  -- geodesic icosphere, radial noise
  x(1 + N(0, noise)) per vertex (5,120 triangles at level 4);
* ``torus(nu, nv, R, r, seed)``  -- bumpy genus-1 torus, radial displacement
  0.03 sin(5u) cos(7v) + N(0, 0.003);
* ``ellipsoid(nlon, nlat, axes, seed)``  -- lat-long ellipsoid with the sum of
  8 random real spherical harmonics (degree <= 6, amplitude 0.02) as a radial
  bump; poles are kept as single vertices of valence ``nlon``;
* ``torus_knot_tube(nu, nv, radius, seed)``  -- (2,3) torus-knot tube;
* ``plane``, ``single_triangle``, ``cube`` -- tiny edge cases of the same
  kind as the reference's input/edgeCases folder.

All functions return ``(V, F)`` with V float64 (n, 3) and F int32 (m, 3),
counter-clockwise outward orientation for closed surfaces.
"""
from __future__ import annotations

import math

import numpy as np


# ---------------------------------------------------------------- OBJ I/O
def write_obj(path, V, F):
    with open(path, "w") as f:
        for p in V:
            f.write("v %.17g %.17g %.17g\n" % (p[0], p[1], p[2]))
        for t in F:
            f.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


def read_obj(path):
    V, F = [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                V.append([float(x) for x in line.split()[1:4]])
            elif line.startswith("f "):
                F.append([int(tok.split("/")[0]) - 1 for tok in line.split()[1:4]])
    if not V or not F:
        raise ValueError("%s: empty or truncated OBJ" % path)
    return np.asarray(V, np.float64), np.asarray(F, np.int32)


# ---------------------------------------------------------------- meshes
def icosphere(level=4, noise=0.01, seed=0):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    F = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    V = [list(np.asarray(p, float) / np.linalg.norm(p)) for p in V]
    for _ in range(level):
        mid = {}
        newF = []

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in mid:
                p = np.asarray(V[a]) + np.asarray(V[b])
                V.append(list(p / np.linalg.norm(p)))
                mid[key] = len(V) - 1
            return mid[key]

        for a, b, c in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            newF += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        F = newF
    V = np.asarray(V, np.float64)
    if noise > 0:
        rng = np.random.default_rng(seed)
        V = V * (1.0 + rng.normal(0.0, noise, size=(len(V), 1)))
    return V, np.asarray(F, np.int32)


def _grid_torus_faces(nu, nv):
    """Quads of an nu x nv periodic grid split into two triangles each."""
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    i, j = i.ravel(), j.ravel()
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    F = np.empty((2 * nu * nv, 3), np.int32)
    F[0::2] = np.stack([a, b, c], 1)
    F[1::2] = np.stack([a, c, d], 1)
    return F


def torus(nu=160, nv=128, R=1.0, r=0.35, seed=1):
    u = 2 * np.pi * np.arange(nu) / nu
    v = 2 * np.pi * np.arange(nv) / nv
    U, W = np.meshgrid(u, v, indexing="ij")
    rng = np.random.default_rng(seed)
    rr = r + 0.03 * np.sin(5 * U) * np.cos(7 * W) + rng.normal(0.0, 0.003, U.shape)
    X = (R + rr * np.cos(W)) * np.cos(U)
    Y = (R + rr * np.cos(W)) * np.sin(U)
    Z = rr * np.sin(W)
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    return V, _grid_torus_faces(nu, nv)


def _real_sph_harm(l, m, theta, phi):
    """Real spherical harmonic Y_lm (unnormalised); theta polar, phi azimuth.

    Associated Legendre P_l^|m|(cos theta) by the standard three-term
    recurrence in l."""
    am = abs(m)
    x = np.cos(theta)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    pmm = np.ones_like(x)
    fact = 1.0
    for _ in range(am):
        pmm = -pmm * fact * s
        fact += 2.0
    if l == am:
        p = pmm
    else:
        pm1 = x * (2 * am + 1) * pmm
        if l == am + 1:
            p = pm1
        else:
            p0, p1 = pmm, pm1
            for ll in range(am + 2, l + 1):
                p2 = ((2 * ll - 1) * x * p1 - (ll + am - 1) * p0) / (ll - am)
                p0, p1 = p1, p2
            p = p1
    if m > 0:
        return p * np.cos(am * phi)
    if m < 0:
        return p * np.sin(am * phi)
    return p


def ellipsoid(nlon=316, nlat=316, axes=(1.0, 0.6, 0.4), n_bumps=8, lmax=6,
              amplitude=0.02, seed=2):
    """Lat-long ellipsoid: nlat latitude bands, nlon longitudes, two poles."""
    rng = np.random.default_rng(seed)
    theta = np.pi * np.arange(1, nlat) / nlat          # nlat-1 rings
    phi = 2 * np.pi * np.arange(nlon) / nlon
    TH, PH = np.meshgrid(theta, phi, indexing="ij")
    th_all = np.concatenate([[0.0], TH.ravel(), [np.pi]])
    ph_all = np.concatenate([[0.0], PH.ravel(), [0.0]])
    bump = np.zeros_like(th_all)
    for _ in range(n_bumps):
        l = int(rng.integers(1, lmax + 1))
        m = int(rng.integers(-l, l + 1))
        c = rng.uniform(-1.0, 1.0)
        y = _real_sph_harm(l, m, th_all, ph_all)
        bump += c * y / max(np.abs(y).max(), 1e-12)
    bump /= max(np.abs(bump).max(), 1e-12)
    scale = 1.0 + amplitude * bump
    a, b, c = axes
    X = a * np.sin(th_all) * np.cos(ph_all) * scale
    Y = b * np.sin(th_all) * np.sin(ph_all) * scale
    Z = c * np.cos(th_all) * scale
    V = np.stack([X, Y, Z], 1)
    nr = nlat - 1
    north, south = 0, 1 + nr * nlon

    def ring(k, j):
        return 1 + k * nlon + (j % nlon)

    F = []
    # the first face avoids the poles (the one-point cut starts at F[0][0])
    for k in range(nr - 1):
        for j in range(nlon):
            a0, a1 = ring(k, j), ring(k, j + 1)
            b0, b1 = ring(k + 1, j), ring(k + 1, j + 1)
            F.append([a0, b0, b1])
            F.append([a0, b1, a1])
    for j in range(nlon):
        F.append([north, ring(0, j), ring(0, j + 1)])
        F.append([south, ring(nr - 1, j + 1), ring(nr - 1, j)])
    return V, np.asarray(F, np.int32)


def torus_knot_tube(nu=2000, nv=512, p=2, q=3, radius=0.15, noise=0.002, seed=4):
    t = 2 * np.pi * np.arange(nu) / nu
    rr = 1.0 + 0.4 * np.cos(q * t)

    def curve(tt):
        r_ = 1.0 + 0.4 * np.cos(q * tt)
        return np.stack([r_ * np.cos(p * tt), r_ * np.sin(p * tt), 0.4 * np.sin(q * tt)], 1)

    C = curve(t)
    dt = 1e-4
    T = curve(t + dt) - curve(t - dt)
    T /= np.linalg.norm(T, axis=1, keepdims=True)
    ref = np.array([0.0, 0.0, 1.0])
    N = np.cross(T, ref)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    B = np.cross(T, N)
    w = 2 * np.pi * np.arange(nv) / nv
    rng = np.random.default_rng(seed)
    rad = radius * (1.0 + rng.normal(0.0, noise, (nu, nv)))
    P = (C[:, None, :] + rad[..., None] * (np.cos(w)[None, :, None] * N[:, None, :]
                                           + np.sin(w)[None, :, None] * B[:, None, :]))
    del rr
    return P.reshape(-1, 3), _grid_torus_faces(nu, nv)


def bumpy_sheet(n=40, amp=0.25, noise=0.01, seed=5):
    """Open disk: n x n grid over [-1, 1]^2 with height
    amp * sin(2x) * cos(3y) plus N(0, noise); alternating diagonals."""
    rng = np.random.default_rng(seed)
    x, y = np.meshgrid(np.linspace(-1.0, 1.0, n), np.linspace(-1.0, 1.0, n), indexing="ij")
    z = amp * np.sin(2.0 * x) * np.cos(3.0 * y) + rng.normal(0.0, noise, x.shape)
    V = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    F = []
    for i in range(n - 1):
        for j in range(n - 1):
            a, b, c, d = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
            if (i + j) % 2 == 0:
                F += [[a, b, c], [a, c, d]]
            else:
                F += [[a, b, d], [b, c, d]]
    return V, np.asarray(F, np.int32)


def plane():
    V = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float64)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    return V, F


def single_triangle():
    V = np.array([[0, 0, 0], [1, 0, 0], [0.3, 0.8, 0]], np.float64)
    return V, np.array([[0, 1, 2]], np.int32)


def cube():
    V = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float64)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    F = []
    for a, b, c, d in quads:
        F += [[a, b, c], [a, c, d]]
    return V, np.asarray(F, np.int32)


def components_mesh():
    """Three components in one mesh: a sphere, a torus and a bumpy sheet
    (the reference cuts each by its own Euler characteristic and lays their
    UV disks out on a grid)."""
    parts = [icosphere(2, 0.01, 0), torus(24, 16, 1.0, 0.35, 1), bumpy_sheet(12, 0.25, 0.01, 5)]
    V, F, off = [], [], 0
    for k, (v, f) in enumerate(parts):
        V.append(np.asarray(v, np.float64) + np.array([3.0 * k, 0.0, 0.0]))
        F.append(np.asarray(f, np.int32) + off)
        off += len(v)
    return np.vstack(V), np.vstack(F).astype(np.int32)


CONFIGS = {
    # the five synthetic workloads, by the reference's own sizes
    "icosphere_5k": lambda: icosphere(4, 0.01, 0),
    "torus_41k": lambda: torus(160, 128, 1.0, 0.35, 1),
    "ellipsoid_199k": lambda: ellipsoid(316, 316, (1.0, 0.6, 0.4), 8, 6, 0.02, 2),
    "knot_2m": lambda: torus_knot_tube(2000, 512, 2, 3, 0.15, 0.002, 4),
    # small members of the same families (parity fixtures)
    "icosphere_320": lambda: icosphere(2, 0.01, 0),
    "icosphere_1k": lambda: icosphere(3, 0.01, 0),
    "ellipsoid_2k": lambda: ellipsoid(32, 32, (1.0, 0.6, 0.4), 8, 6, 0.02, 2),
    "ellipsoid_20k": lambda: ellipsoid(100, 100, (1.0, 0.6, 0.4), 8, 6, 0.02, 2),
    "torus_768": lambda: torus(24, 16, 1.0, 0.35, 1),
    "sheet_3k": lambda: bumpy_sheet(40, 0.25, 0.01, 5),
    "cube": cube,
    "plane": plane,
    "triangle": single_triangle,
    "components": components_mesh,
}
