"""The oracle port against golden vectors produced by the reference itself
(tests/golden/make_golden.py): bit-exact random streams, particle states,
potentials.  CPU only."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def port_lib(built):
    from mag2d_cases import load_port

    return load_port()


def _meta(d):
    return json.loads(str(d["meta"]))


def test_rng_streams_match_reference(port_lib):
    from mag2d_cases import Port

    g = np.load(GOLDEN / "rng.npz")
    cfg = dict(coord="CARTESIAN", geometry="EMPTY", x_sampl=5, z_sampl=5, selfconsistent=0, rf=0)
    mask = np.zeros((5, 5), np.int8)
    p = Port(cfg, [dict(name="E", mass=9.11e-31, charge=-1.6e-19, dt=1e-11, temperature=1e4)], [], mask,
             np.zeros((5, 5)))
    for seed in (1, 1234, 4242):
        p.L.orc_seed(p.h, seed)
        assert np.array_equal(p.rng(0, 1000), g[f"uni_{seed}"])
        assert np.array_equal(p.rng(1, 4000), g[f"rnor_{seed}"])
        assert np.array_equal(p.rng(2, 4000), g[f"rexp_{seed}"])
        assert np.array_equal(p.rng(3, 500), g[f"iuni_{seed}"])
        assert np.array_equal(p.rng(4, 500), g[f"rot_{seed}"])
        assert np.array_equal(p.rng(5, 500, 0.75 * np.pi), g[f"deflect_{seed}"])


def test_rng_distribution_kats(port_lib):
    """Known-answer properties of the reference's generators (tests/test_deflect.cpp,
    the isotropy and Maxwellian checks of tests/rot_test.cpp and tests/maxwell_test.cpp)."""
    g = np.load(GOLDEN / "rng.npz")
    rnor = g["rnor_1234"]
    assert abs(rnor.mean()) < 4 / np.sqrt(len(rnor)) and abs(rnor.std() - 1) < 0.05
    rexp = g["rexp_1234"]
    assert abs(rexp.mean() - 1) < 0.05
    rot = g["rot_1234"].reshape(-1, 3)
    assert np.allclose(np.linalg.norm(rot, axis=1), 1.0, atol=1e-12)
    assert np.abs(rot.mean(axis=0)).max() < 0.1
    d = g["deflect_1234"].reshape(-1, 3)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-9)  # deflect preserves |v|
    assert np.allclose(d[:, 0], np.cos(0.75 * np.pi), atol=1e-9)  # by the requested angle


STEP_CASES = sorted(p.name for p in GOLDEN.glob("step_*.npz"))


@pytest.mark.parametrize("fname", STEP_CASES)
def test_step_matches_reference(port_lib, fname, tmp_path):
    from mag2d_cases import Port

    d = np.load(GOLDEN / fname)
    m = _meta(d)
    loaded = None
    if m["has_fields"]:
        nx, nz, dx, dz = d["f_grid"]
        loaded = (int(nx), int(nz), dx, dz, 0.0, 0.0, d["f_u"], d["f_urf"])
    port = Port(m["cfg"], m["species"], m["inter"], d["mask"], d["voltage"], seed=m["seed"], loaded_fields=loaded)
    ns = len(m["species"])
    for s in range(ns):
        if f"init_{s}" in d:
            port.set_particles(s, *d[f"init_{s}"])
    if m["initscript"]:
        (tmp_path / "init.txt").write_text(m["initscript"])
        port.run_initscript(tmp_path / "init.txt")
    port.advance_init()
    for s in range(ns):
        assert np.array_equal(port.particles(s), d[f"p_init_{s}"]), (fname, "init", s)
    done = 0
    for k in m["snaps"]:
        port.advance(k - done)
        done = k
        for s in range(ns):
            got, want = port.particles(s), d[f"p_{k}_{s}"]
            assert got.shape == want.shape, (fname, k, s)
            assert np.array_equal(got, want), (fname, k, s, np.nanmax(np.abs(got - want)))
    assert np.array_equal(port.field(0), d["u"])
    if not m["has_fields"]:  # with loaded fields the reference leaves rho uninitialised (pic.cpp:163)
        assert np.array_equal(port.field(2), d["rho"])


@pytest.mark.parametrize("tag", ["cyl", "cart"])
def test_u_smooth_matches_reference(port_lib, tag):
    """Fields::u_smooth (fields.cpp:28-111) bit for bit, flat-index wrap of the
    last column included; the node whose stencil reads one element past the
    reference's array (row nx-2, column nz-1) is left out of the comparison."""
    d = np.load(GOLDEN / "u_smooth.npz")
    u, want = d[f"u_{tag}"], d[f"smooth_{tag}"]
    out = np.zeros_like(u)
    port_lib.orc_u_smooth(u.shape[0], u.shape[1], u.ctypes.data, out.ctypes.data)
    keep = np.ones(u.shape, dtype=bool)
    keep[-2, -1] = False
    assert np.array_equal(out[keep], want[keep])
    # the untouched rows and first column stay as they were
    assert np.array_equal(out[0], u[0]) and np.array_equal(out[-1], u[-1]) and np.array_equal(out[:, 0], u[:, 0])
    # the wrap: the last column reads column 0 of the next row
    i, j, nz = 5, u.shape[1] - 1, u.shape[1]
    f = u.reshape(-1)
    k = i * nz + j
    s = (f[k] + f[k - nz] * 0.5 + f[k + nz] * 0.5 + f[k - 1] * 0.5 + f[k + 1] * 0.5 + f[k - nz - 1] * 0.25
         + f[k + nz - 1] * 0.25 + f[k - nz + 1] * 0.25 + f[k + nz + 1] * 0.25) / 4.0
    assert want[i, j] == s


@pytest.mark.parametrize("fname", sorted(p.name for p in GOLDEN.glob("solve_*.npz")))
def test_poisson_solve_matches_reference(port_lib, fname):
    from mag2d_cases import Port

    d = np.load(GOLDEN / fname)
    m = _meta(d)
    port = Port(m["cfg"], m["species"], [], d["mask"], d["voltage"])
    u = port.solve(d["rho"])
    assert np.array_equal(u, d["u"])


@pytest.mark.parametrize("fname", sorted(p.name for p in GOLDEN.glob("solve_*.npz")))
def test_poisson_solve_independent_check(fname):
    """The reference's linear system (fields.cpp:136-312) solved by SciPy's
    SuperLU agrees with the golden potential to 1e-11 (pins the banded LU used
    in place of UMFPACK)."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    from mag2d_cases import EPS0, full_config

    d = np.load(GOLDEN / fname)
    m = _meta(d)
    c = full_config(m["cfg"])
    mask, volt, rho = d["mask"], d["voltage"], d["rho"]
    nx, nz = mask.shape
    dx, dz = float(c["x_max"]) / (nx - 1), float(c["z_max"]) / (nz - 1)
    cyl = c["coord"] == "CYLINDRICAL"
    rows, cols, vals = [], [], []
    b = np.zeros(nx * nz)
    for i in range(nx):
        for j in range(nz):
            k = i * nz + j
            if mask[i, j] in (0, 1):
                rows.append(k), cols.append(k), vals.append(1.0)
                b[k] = volt[i, j] if mask[i, j] == 0 else 0.0
                continue
            if cyl and i == 0:
                k2, k3 = 1 / dz ** 2, 1 / (dx * dx * 0.25)
                st = [(k - 1, k2), (k, -2 * k2 - k3), (k + 1, k2), (k + nz, k3)]
                b[k] = rho[i, j] * (-1.0 / EPS0 / (np.pi * dx * dx * 0.25 * dz) * float(c["macroparticle_factor"]))
            elif cyl:
                k1, k2, k3 = (i - 0.5) / (dx * dx * i), 1 / dz ** 2, (i + 0.5) / (dx * dx * i)
                st = [(k - nz, k1), (k - 1, k2), (k, -2 * k2 - k1 - k3), (k + 1, k2), (k + nz, k3)]
                b[k] = rho[i, j] * (-1.0 / EPS0 / (np.pi * dx * dx * 2.0 * i * dz) * float(c["macroparticle_factor"]))
            else:
                V = float(c["n_particles_total"]) / float(c["density_total"])
                dV = V / ((nx - 1) * (nz - 1))
                st = [(k - nz, 1.0), (k - 1, 1.0), (k, -4.0), (k + 1, 1.0), (k + nz, 1.0)]
                b[k] = rho[i, j] * (-dx * dx / EPS0 / dV)
            for cc, v in st:
                rows.append(k), cols.append(cc), vals.append(v)
    A = sp.csc_matrix((vals, (rows, cols)), shape=(nx * nz, nx * nz))
    lu = spl.splu(A)
    u = lu.solve(b)
    for _ in range(3):  # iterative refinement: SuperLU alone leaves ~1e-8 residuals on these systems
        u = u + lu.solve(b - A @ u)
    assert np.abs(u.reshape(nx, nz) - d["u"]).max() <= 1e-11 * np.abs(d["u"]).max()


def test_fixed_point_deposit_properties(port_lib):
    """The quantised CIC deposit conserves charge exactly (2^40 per particle)
    and stays within 2^-20 per weight of the reference's FP64 weights."""
    from mag2d_cases import deposit_fixed, to_fixed

    rng = np.random.default_rng(1)
    n, nx, nz = 5000, 17, 33
    xf = to_fixed(rng.random(n) * (nx - 1))
    zf = to_fixed(rng.random(n) * (nz - 1))
    xg, zg = xf / 2.0 ** 20, zf / 2.0 ** 20
    acc = deposit_fixed(nx, nz, xf, zf)
    assert acc.sum() == n << 40
    ref = np.zeros((nx, nz))
    i, j = np.minimum(np.floor(xg).astype(int), nx - 2), np.minimum(np.floor(zg).astype(int), nz - 2)
    u, v = xg - i, zg - j
    np.add.at(ref, (i, j), (1 - u) * (1 - v))
    np.add.at(ref, (i + 1, j), u * (1 - v))
    np.add.at(ref, (i, j + 1), (1 - u) * v)
    np.add.at(ref, (i + 1, j + 1), u * v)
    counts = np.zeros((nx, nz))
    for di in (0, 1):
        for dj in (0, 1):
            np.add.at(counts, (i + di, j + dj), 1)
    assert np.all(np.abs(acc / 2.0 ** 40 - ref) <= counts * 2.0 ** -19)
    # order independence: any permutation gives identical integers
    perm = rng.permutation(n)
    assert np.array_equal(deposit_fixed(nx, nz, xf[perm], zf[perm]), acc)


def test_particle_file_matches_reference_save(built):
    """The library reads the file BaseSpecies::save wrote (exact doubles) and
    writes the same bytes for the same particles (record padding aside)."""
    import mag2d_gb300 as m

    d = np.load(GOLDEN / "particles.npz")
    f = m.read_particle_file(GOLDEN / "particles_ref.dat")
    assert f["total"] == len(d["x"])
    for k in ("x", "z", "vx", "vy", "vz"):
        assert np.array_equal(f[k], d[k]), k
    assert not f["y"].any() and not f["time_to_death"].any()
    import tempfile

    with tempfile.TemporaryDirectory() as t:
        p = Path(t) / "ours.dat"
        m.write_particle_file(p, d["x"], d["z"], d["vx"], d["vy"], d["vz"], total=len(d["x"]))
        ours, ref = p.read_bytes(), (GOLDEN / "particles_ref.dat").read_bytes()
    assert len(ours) == len(ref) == 8 + 64 * len(d["x"])
    assert ours[:8] == ref[:8]
    for i in range(len(d["x"])):
        a = 8 + 64 * i
        assert ours[a:a + 57] == ref[a:a + 57], i  # 7 doubles and the empty flag


def test_source_golden_fixture():
    """The reference's source box file and inflow curve (make_golden.py source):
    N / src_fact box particles inside the box, and a domain filling toward
    density * V (the source's purpose) without overshoot."""
    g = np.load(GOLDEN / "source.npz", allow_pickle=True)
    meta = json.loads(str(g["meta"]))
    cfg, sp = meta["cfg"], meta["species"][0]
    raw = (GOLDEN / "source_ref.dat").read_bytes()
    n = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    rec = np.frombuffer(raw[4:], dtype=np.float64).reshape(n, 8)
    V = cfg["n_particles_total"] / cfg["density_total"]
    assert n == int(sp["density"] * V / cfg["src_fact"])
    bx, bz = cfg["x_max"] / cfg["src_fact"], cfg["z_max"] / cfg["src_fact"]
    assert np.all((rec[:, 0] >= 0) & (rec[:, 0] < bx) & (rec[:, 2] >= 0) & (rec[:, 2] < bz))
    vsig = np.sqrt(1.380662e-23 * sp["temperature"] / sp["mass"])
    assert abs(rec[:, 3].std() / vsig - 1) < 0.1 and abs(rec[:, 5].std() / vsig - 1) < 0.1
    live = g["live"]
    assert np.all(np.diff(live) > 0) and live[-1] < 1.05 * sp["density"] * V


def test_field3d_oracle_pinned():
    """The 3D oracle's accumulate / interpolate / grad against the reference's
    own Field3D header (golden vectors of oracle/ref/field3d_harness.cpp)."""
    import sys

    sys.path.insert(0, str(GOLDEN.parents[1] / "oracle"))
    import mag3d_oracle as o

    g = np.load(GOLDEN / "field3d.npz")
    shape, d = tuple(int(v) for v in g["shape"]), tuple(g["d"])
    rho = o.accumulate(shape, d, g["charge"], g["x"], g["y"], g["z"])
    assert np.abs(rho - g["rho"]).max() <= 1e-13 * np.abs(g["rho"]).max()
    it = o.interpolate(g["u"], d, g["x"], g["y"], g["z"])
    assert np.abs(it - g["interp"]).max() <= 1e-13 * np.abs(g["u"]).max()
    gr = o.grad(g["u"], d, g["x"], g["y"], g["z"])
    assert np.abs(gr - g["grad"]).max() <= 1e-13 * np.abs(g["grad"]).max()


def test_oracle3d_solve_satisfies_the_7_point_equations():
    pytest.importorskip("scipy")
    import sys

    sys.path.insert(0, str(GOLDEN.parents[1] / "oracle"))
    import mag3d_oracle as o

    shape, d = (11, 9, 13), (1e-3, 1.2e-3, 0.9e-3)
    fixed, volt = o.geometry3d(*shape)
    rho = np.random.default_rng(3).normal(0, 1e-8, shape)
    u = o.solve(rho, fixed, volt, d)
    assert np.array_equal(u[fixed], volt[fixed])
    lap = np.zeros(shape)
    for a in range(3):
        lap[1:-1, 1:-1, 1:-1] += (np.roll(u, 1, a) - 2 * u + np.roll(u, -1, a))[1:-1, 1:-1, 1:-1] / d[a] ** 2
    res = (lap + rho / o.EPS0)[~fixed]
    assert np.abs(res).max() <= 1e-9 * np.abs(rho / o.EPS0).max()
