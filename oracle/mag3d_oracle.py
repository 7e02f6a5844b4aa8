"""CPU restatement of the 3D Cartesian path — test infrastructure only.

Only the tests import this module, as the checker of the GPU 3D run
(mag3d_* of libmag2d_gpu.so); nothing in the product calls it.

It follows the reference's 3D code (src/Field3D.hpp:40-163,
src/fields3d.cpp:11-101, src/species3d.cpp:3-94):
  * geometry3d     Geometry::Geometry: box faces fixed at 0 V, the centre node
                   (the Quadrupole placeholder, fields3d.hpp:26-35) at 1 V
  * accumulate     Field3D::accumulate (trilinear CIC, FP64)
  * deposit_fixed  the GPU's integer form of it on fixed-point positions
                   (14-bit weights per axis), which it must match bit for bit
  * grad           Field3D::grad / grad_component (staggered differences,
                   trilinear), with the domain extent as the clamp bound
  * solve          the 7-point problem of Solver::matrix_init with the grid
                   spacings, -lap(u) = rho / eps0 on the free nodes, by a
                   sparse direct solve
  * step           Species<CARTESIAN3D>::advance: half acceleration, Boris
                   rotation, half acceleration, move, FREE / PERIODIC
                   boundary, is_free (8 corners)
The reference's 3D code does not build as shipped, so only Field3D's
accumulate / interpolate / grad are pinned against it (golden vectors from
oracle/ref/field3d_harness.cpp); the solve and the step are parity-unpinned
restatements of the mathematics.
"""
from __future__ import annotations

import numpy as np

EPS0 = 8.854187817e-12  # src/param.cpp:8-10
FRAC_BITS = 20
DEP_BITS = 14


def geometry3d(nx: int, ny: int, nz: int):
    """Fixed-node mask (True = Dirichlet) and voltages."""
    fixed = np.zeros((nx, ny, nz), dtype=bool)
    fixed[0, :, :] = fixed[-1, :, :] = True
    fixed[:, 0, :] = fixed[:, -1, :] = True
    fixed[:, :, 0] = fixed[:, :, -1] = True
    volt = np.zeros((nx, ny, nz))
    c = (nx // 2, ny // 2, nz // 2)
    fixed[c] = True
    volt[c] = 1.0
    return fixed, volt


def cellfree(fixed: np.ndarray) -> np.ndarray:
    """t_grid::is_free per cell: at least one of its 8 corners is free."""
    f = ~fixed
    return (f[:-1, :-1, :-1] | f[1:, :-1, :-1] | f[:-1, 1:, :-1] | f[1:, 1:, :-1] |
            f[:-1, :-1, 1:] | f[1:, :-1, 1:] | f[:-1, 1:, 1:] | f[1:, 1:, 1:])


def accumulate(shape, d, charge, x, y, z) -> np.ndarray:
    """Field3D::accumulate of every (charge, x, y, z) into a zero grid."""
    rho = np.zeros(shape)
    for q, px, py, pz in zip(np.broadcast_to(charge, np.shape(x)), x, y, z):
        X, Y, Z = px / d[0], py / d[1], pz / d[2]
        i, j, k = int(X), int(Y), int(Z)
        u, v, w = X - i, Y - j, Z - k
        for di, wi in ((0, 1 - u), (1, u)):
            for dj, wj in ((0, 1 - v), (1, v)):
                for dk, wk in ((0, 1 - w), (1, w)):
                    rho[i + di, j + dj, k + dk] += wi * wj * wk * q
    return rho


def interpolate(f: np.ndarray, d, x, y, z) -> np.ndarray:
    """Field3D::interpolate at every point."""
    out = np.zeros(len(x))
    for p, (px, py, pz) in enumerate(zip(x, y, z)):
        X, Y, Z = px / d[0], py / d[1], pz / d[2]
        i, j, k = int(X), int(Y), int(Z)
        u, v, w = X - i, Y - j, Z - k
        g = f[i:i + 2, j:j + 2, k:k + 2]
        out[p] = _trilin(g, u, v, w)
    return out


def _trilin(g, u, v, w):
    return ((1 - u) * (1 - v) * (1 - w) * g[0, 0, 0] + u * (1 - v) * (1 - w) * g[1, 0, 0] +
            (1 - u) * v * (1 - w) * g[0, 1, 0] + u * v * (1 - w) * g[1, 1, 0] +
            (1 - u) * (1 - v) * w * g[0, 0, 1] + u * (1 - v) * w * g[1, 0, 1] +
            (1 - u) * v * w * g[0, 1, 1] + u * v * w * g[1, 1, 1])


def grad(f: np.ndarray, d, x, y, z) -> np.ndarray:
    """Field3D::grad at every point: (n, 3)."""
    shape = f.shape
    ext = [(shape[a] - 1) * d[a] for a in range(3)]
    out = np.zeros((len(x), 3))
    for p, pos in enumerate(zip(x, y, z)):
        for a in range(3):
            e = [0, 0, 0]
            e[a] = 1
            c = [min(max(pos[b] / d[b], 0.5 * e[b]), ext[b] / d[b] - 0.5 * e[b]) for b in range(3)]
            idx = [int(c[b] + 0.5 * e[b]) for b in range(3)]
            fr = [c[b] + 0.5 * e[b] - idx[b] for b in range(3)]
            g = np.zeros((2, 2, 2))
            for di in range(2):
                for dj in range(2):
                    for dk in range(2):
                        i, j, k = idx[0] + di, idx[1] + dj, idx[2] + dk
                        if fr[0] == 0 and di == 1 or fr[1] == 0 and dj == 1 or fr[2] == 0 and dk == 1:
                            continue  # zero weight (the reference reads past the array there)
                        g[di, dj, dk] = f[i, j, k] - f[i - e[0], j - e[1], k - e[2]]
            out[p, a] = _trilin(g, *fr) / d[a]
    return out


def to_fixed(v, h):
    return np.rint(np.asarray(v, dtype=np.float64) / h * (1 << FRAC_BITS)).astype(np.int64)


def deposit_fixed(shape, xf, yf, zf) -> np.ndarray:
    """The GPU deposit: 8 int64 corner weights per particle (2^42 in total)."""
    nx, ny, nz = shape
    rho = np.zeros(shape, dtype=np.int64)
    one = 1 << DEP_BITS
    sh = FRAC_BITS - DEP_BITS
    xf, yf, zf = (np.asarray(a, dtype=np.int64) for a in (xf, yf, zf))
    i = np.minimum(xf >> FRAC_BITS, nx - 2)
    j = np.minimum(yf >> FRAC_BITS, ny - 2)
    k = np.minimum(zf >> FRAC_BITS, nz - 2)
    U = (xf - (i << FRAC_BITS)) >> sh
    V = (yf - (j << FRAC_BITS)) >> sh
    W = (zf - (k << FRAC_BITS)) >> sh
    for di, wi in ((0, one - U), (1, U)):
        for dj, wj in ((0, one - V), (1, V)):
            for dk, wk in ((0, one - W), (1, W)):
                np.add.at(rho, (i + di, j + dj, k + dk), wi * wj * wk)
    return rho


def solve(rho: np.ndarray, fixed: np.ndarray, volt: np.ndarray, d) -> np.ndarray:
    """-lap(u) = rho / eps0 on the free nodes, u = volt on the fixed ones."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spl

    shape = rho.shape
    n = rho.size
    free = ~fixed.reshape(-1)
    idx = -np.ones(n, dtype=np.int64)
    idx[free] = np.arange(free.sum())
    strides = (shape[1] * shape[2], shape[2], 1)
    coords = np.unravel_index(np.arange(n), shape)
    rows, cols, vals = [], [], []
    b = (rho.reshape(-1) / EPS0)[free].copy()
    u_fix = volt.reshape(-1)
    fq = np.flatnonzero(free)
    rows.append(idx[fq])
    cols.append(idx[fq])
    vals.append(np.full(len(fq), sum(2.0 / d[a] ** 2 for a in range(3))))
    for a in range(3):
        w = 1.0 / d[a] ** 2
        for s in (-1, 1):
            c = coords[a][fq] + s
            ok = (c >= 0) & (c < shape[a])
            q = fq[ok]
            nb = q + s * strides[a]
            fnb = free[nb]
            rows.append(idx[q[fnb]])
            cols.append(idx[nb[fnb]])
            vals.append(np.full(fnb.sum(), -w))
            np.add.at(b, idx[q[~fnb]], w * u_fix[nb[~fnb]])
    A = sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(free.sum(), free.sum()))
    lu = spl.splu(A.tocsc())
    x = lu.solve(b)
    for _ in range(2):
        x = x + lu.solve(b - A @ x)
    u = u_fix.copy()
    u[free] = x
    return u.reshape(shape)


def step(state: dict, E, B, qm: float, dt: float, ext, periodic: bool, free_cell: np.ndarray, d) -> dict:
    """One Species<CARTESIAN3D>::advance of the live particles (FP64).

    state: x, y, z, vx, vy, vz, alive (arrays); E(x, y, z) -> (n, 3);
    B = (Bx, By, Bz)."""
    x, y, z = state["x"], state["y"], state["z"]
    v = np.stack([state["vx"], state["vy"], state["vz"]], axis=1)
    alive = state["alive"].copy()
    e = E(x, y, z)
    h = qm * dt / 2.0
    v = v + e * h
    t = np.asarray(B, dtype=np.float64) * h
    if np.any(t != 0):
        s = 2.0 * t / (1.0 + t @ t)
        vp = v + np.cross(v, t)
        v = v + np.cross(vp, s)
    v = v + e * h
    pos = np.stack([x, y, z], axis=1) + v * dt
    ext = np.asarray(ext)
    out = np.any((pos < 0) | (pos > ext), axis=1)
    if periodic:
        pos = np.mod(pos, ext)
        out[:] = False
    alive &= ~out
    cells = np.minimum((pos / np.asarray(d)).astype(np.int64), np.asarray(free_cell.shape) - 1)
    cells = np.maximum(cells, 0)
    ok = free_cell[cells[:, 0], cells[:, 1], cells[:, 2]]
    alive &= ok
    return {"x": pos[:, 0], "y": pos[:, 1], "z": pos[:, 2], "vx": v[:, 0], "vy": v[:, 1], "vz": v[:, 2],
            "alive": alive}


def leapfrog_start(state: dict, E, B, qm: float, dt: float) -> dict:
    """Half backward rotation and half backward acceleration (advance_boris_init)."""
    v = np.stack([state["vx"], state["vy"], state["vz"]], axis=1)
    h = -qm * dt / 2.0
    t = np.asarray(B, dtype=np.float64) * (-0.5 * qm * dt / 2.0)
    if np.any(t != 0):
        s = 2.0 * t / (1.0 + t @ t)
        vp = v + np.cross(v, t)
        v = v + np.cross(vp, s)
    v = v + E(state["x"], state["y"], state["z"]) * h
    return dict(state, vx=v[:, 0], vy=v[:, 1], vz=v[:, 2])
