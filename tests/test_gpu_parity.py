"""GPU parity tests: the CUDA path through the C ABI against the oracle port.

Tolerances:
  * deposit        — bit-exact against the oracle's fixed-point CIC deposit
  * Poisson solve  — |u_gpu - u_oracle|_inf <= 1e-9 |u_oracle|_inf
  * trajectories   — every position within 1e-5 of the domain size after 1000
                     steps with collisions off (FP32 state against the FP64
                     oracle); velocities within the bounds each test states
  * MCC            — collision counts within 3 sigma of the expected count and a
                     two-sample KS test on energies at p > 0.01
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def _port_for(m, cfg, species, inter, cpath, seed=1, loaded=None):
    from mag2d_cases import Port

    mask, volt = m.config_geometry(cpath)
    return Port(cfg, species, inter, mask, volt, seed=seed, loaded_fields=loaded)


def _match(g, o):
    """Map GPU particles (by id) onto oracle slots (slot i holds input i)."""
    live = o[:, 7] == 0
    ids = g["id"].astype(np.int64)
    common = np.intersect1d(ids, np.flatnonzero(live))
    pos = {int(k): i for i, k in enumerate(ids)}
    sel = np.array([pos[int(k)] for k in common], dtype=np.int64)
    return common, sel, live


# ---------------------------------------------------------------------------
# Poisson: FP32 multigrid + FP64 refinement against the oracle's direct solve
@pytest.mark.parametrize("geom", [
    dict(coord="CYLINDRICAL", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3, r_sampl=65, z_sampl=129),
    dict(coord="CYLINDRICAL", geometry="PENNING_SIMPLE", r_max=1.2e-2, z_max=7.5e-2, r_sampl=33, z_sampl=129),
    dict(coord="CYLINDRICAL", geometry="PENNING", r_max=1.2e-2, z_max=7.5e-2, r_sampl=49, z_sampl=97),
    dict(coord="CARTESIAN", geometry="RF_22PT", x_max=2e-2, z_max=2e-2, x_sampl=129, z_sampl=129),
    dict(coord="CARTESIAN", geometry="PROBE", x_max=2e-2, z_max=2e-2, x_sampl=65, z_sampl=65, probe_radius=1e-3),
    dict(coord="CARTESIAN", geometry="EMPTY", x_max=2e-2, z_max=2e-2, x_sampl=50, z_sampl=50, extern_field=300.0),
], ids=["penning_endcap", "penning_simple", "penning", "rf22pt", "probe", "empty_sor"])
@pytest.mark.parametrize("direct", [-1, 1, "fp64"], ids=["multigrid", "inverse", "multigrid_fp64"])
def test_poisson_matches_direct_solve(m, tmp_path, geom, direct):
    """The three solvers of a small grid: the FP32 multigrid with FP64
    refinement, the product with the precomputed inverse of the operator
    (whose columns are multigrid solves of unit right-hand sides) and the
    all-FP64 multigrid."""
    from mag2d_cases import QE, write_config, write_species_conf

    cfg = dict(selfconsistent=1, rf=0, do_plot=0, macroparticle_factor=100.0, **geom)
    species = [dict(name="E", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, temperature=1e4, density=1e13)]
    cpath = write_config(cfg, tmp_path / "c.txt")
    spath = write_species_conf(species, [], tmp_path / "s.txt")
    fp64 = direct == "fp64"
    direct = -1 if fp64 else direct
    pic = m.Pic(cpath, spath, seed=1, direct_solve=direct, multigrid_fp64=int(fp64))
    port = _port_for(m, cfg, species, [], cpath)
    rng = np.random.default_rng(5)
    nx, nz = pic.shape
    # a space charge of ~1e13 m^-3 electrons: -q * weights of ~10 macro particles per node
    rho = -QE * 10 * rng.random((nx, nz))
    info = pic.field.boundary_solve(rho)
    u_gpu = pic.field.u
    u_ref = port.solve(rho)
    err = np.abs(u_gpu - u_ref).max() / np.abs(u_ref).max()
    assert info["status"] == 0, info
    assert (info["iterations"] == 0) == (direct == 1), info  # the inverse takes no iterations
    assert err <= 1e-9, (err, info)
    pic.close()


def test_inverse_solve_matches_multigrid_in_a_run(m, tmp_path):
    """A self-consistent Penning run (sparse charge: most right-hand-side
    entries zero, so most columns of the inverse are skipped): the potential
    after every one of 20 steps agrees with the multigrid run within 1e-9
    relative, and two runs with the inverse are bit-identical."""
    from cases import penning_segments

    c = penning_segments(tmp_path, n=2000)
    us = {}
    for tag, direct in (("mg", -1), ("inv", 1), ("inv2", 1)):
        pic = m.Pic(c[3], c[4], c[5], seed=3, direct_solve=direct)
        pic.advance_init()
        seq = []
        for _ in range(20):
            pic.advance(1)
            seq.append(pic.field.u.copy())
        us[tag] = np.array(seq)
        pic.close()
    scale = np.abs(us["mg"]).max()
    assert np.abs(us["inv"] - us["mg"]).max() <= 1e-9 * scale
    assert np.array_equal(us["inv"], us["inv2"])


def _faces_of(u, dx, dz):
    """Field2D::grad's staggered faces of u with the end faces repeated, FP32 (faces_pass)."""
    dx_, dz_ = -(u[1:] - u[:-1]) * (1.0 / dx), -(u[:, 1:] - u[:, :-1]) * (1.0 / dz)
    ex = np.concatenate([dx_[:1], dx_, dx_[-1:]], axis=0).astype(np.float32)
    ez = np.concatenate([dz_[:, :1], dz_, dz_[:, -1:]], axis=1).astype(np.float32)
    return ex, ez


def _direct_solve(A, b):
    spl = pytest.importorskip("scipy.sparse.linalg")
    lu = spl.splu(A.tocsc())
    u = lu.solve(b)
    for _ in range(3):  # iterative refinement: SuperLU alone leaves ~1e-8 residuals on these systems
        u = u + lu.solve(b - A @ u)
    return u


def test_poisson_multiblock_matches_direct_solve(m, tmp_path):
    """A grid above the one-block size (257 x 513 = 131841 nodes): the solve
    runs on one block per SM under a cooperative launch with its coarse levels
    on block 0; the potential agrees with a sparse direct solve of the
    reference's system within 1e-9 relative."""
    pytest.importorskip("scipy")
    from mag2d_cases import QE, poisson_system, write_config, write_species_conf

    cfg = dict(coord="CYLINDRICAL", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3, r_sampl=257, z_sampl=513,
               selfconsistent=1, rf=0, do_plot=0, macroparticle_factor=100.0)
    species = [dict(name="E", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, temperature=1e4, density=1e13)]
    cpath = write_config(cfg, tmp_path / "c.txt")
    spath = write_species_conf(species, [], tmp_path / "s.txt")
    pic = m.Pic(cpath, spath, seed=1)
    mask, volt = m.config_geometry(cpath)
    nx, nz = pic.shape
    rng = np.random.default_rng(5)
    for trial in range(2):
        rho = -QE * 10 * rng.random((nx, nz))
        info = pic.field.boundary_solve(rho)
        u_gpu = pic.field.u
        A, b = poisson_system(cfg, mask, volt, rho)
        u_ref = _direct_solve(A, b).reshape(nx, nz)
        err = np.abs(u_gpu - u_ref).max() / np.abs(u_ref).max()
        assert info["status"] == 0 and info["levels"] > 3, info
        assert err <= 1e-9, (trial, err, info)
        # the face field the particles read, written by the pass that confirms convergence
        ex, ez = pic.field.faces
        fx, fz = _faces_of(u_gpu, pic.dx, pic.dz)
        assert np.array_equal(ex, fx) and np.array_equal(ez, fz)
    pic.close()


def test_poisson_large_grid_residual(m, tmp_path):
    """The 1025 x 2049 grid of the large single instance: the FP64 residual of
    the returned potential in the reference's own system, Jacobi-scaled, is
    below 1e-10 of max|u| (the solve's stopping rule, checked independently)."""
    pytest.importorskip("scipy")
    from cases import penning_large
    from mag2d_cases import QE, poisson_system

    cfg, species, inter, cpath, spath, _ = penning_large(tmp_path, make_particles=False)
    pic = m.Pic(cpath, spath, seed=1, poisson_tol=1e-10)
    mask, volt = m.config_geometry(cpath)
    nx, nz = pic.shape
    rng = np.random.default_rng(6)
    rho = -QE * 50 * rng.random((nx, nz))
    info = pic.field.boundary_solve(rho)
    u = pic.field.u.reshape(-1)
    A, b = poisson_system(cfg, mask, volt, rho)
    r = b - A @ u
    res = np.abs(r / A.diagonal()).max() / np.abs(u).max()
    assert info["status"] == 0, info
    assert res <= 1e-10, (res, info)
    ex, ez = pic.field.faces
    fx, fz = _faces_of(u.reshape(nx, nz), pic.dx, pic.dz)
    assert np.array_equal(ex, fx) and np.array_equal(ez, fz)
    pic.close()


# ---------------------------------------------------------------------------
def test_deposit_bit_exact(m, tmp_path):
    from cases import penning_rz
    from mag2d_cases import deposit_fixed, to_fixed

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=50_000)
    pic = m.Pic(cpath, spath, seed=1)
    sp = pic.speclist[0]
    sp.set_particles(*parts)
    pic.deposit()
    got = sp.rho_fixed()
    xg = to_fixed((parts[0] - pic.x_min) / pic.dx)
    zg = to_fixed((parts[1] - pic.z_min) / pic.dz)
    want = deposit_fixed(pic.shape[0], pic.shape[1], xg, zg)
    assert np.array_equal(got, want)
    # every particle contributes exactly 2^40
    assert got.sum() == len(xg) << 40
    pic.close()


# ---------------------------------------------------------------------------
def _trajectory_case(m, tmp_path, make, nsteps, n, species_index, track_r=None, **kw):
    """GPU and oracle after nsteps from the same particles; with track_r = (xc, zc)
    the oracle is stepped one step at a time and the largest distance of each
    particle from (xc, zc) along its orbit is returned as well."""
    out = make(tmp_path, n=n, **kw)
    cfg, species, inter, cpath, spath, parts = out[:6]
    loaded = out[6] if len(out) > 6 else None
    pic = m.Pic(cpath, spath, seed=3)
    pic.speclist[species_index].set_particles(*parts)
    pic.advance_init()
    pic.advance(nsteps)
    pic.sync()
    g = pic.speclist[species_index].particles()
    port = _port_for(m, cfg, species, inter, cpath, seed=3, loaded=loaded)
    port.set_particles(species_index, *parts)
    port.advance_init()
    rmax = None
    if track_r is None:
        port.advance(nsteps)
    else:
        rmax = np.zeros(n)
        for _ in range(nsteps):
            port.advance(1)
            o = port.particles(species_index)
            rmax = np.maximum(rmax, np.hypot(o[:, 0] - track_r[0], o[:, 2] - track_r[1]))
    o = port.particles(species_index)
    pic.close()
    return g, o, rmax


def _trajectory_errors(g, o, lx, lz):
    """Per matched particle: position error relative to the domain size, and
    velocity error |dv| relative to the particle's own speed and to v_rms."""
    common, sel, live = _match(g, o)
    assert len(common) >= live.sum() - 2
    ep = np.maximum(np.abs(g["x"][sel] - o[common, 0]) / lx, np.abs(g["z"][sel] - o[common, 2]) / lz)
    vg = np.stack([g["vx"][sel], g["vy"][sel], g["vz"][sel]], axis=1)
    vo = o[common][:, 3:6]
    dv = np.linalg.norm(vg - vo, axis=1)
    vmag = np.linalg.norm(vo, axis=1)
    vrms = np.sqrt((vo ** 2).sum(axis=1).mean())
    return common, ep, dv / vmag, dv / vrms


def test_penning_trajectories_1000_steps(m, tmp_path):
    """Self-consistent Penning trap (C0 grid), 2000 electrons, 1000 steps with
    collisions off: every position within 1e-5 of the domain size of the
    oracle's (measured max 1e-6).  Velocities: |dv|/|v| <= 5e-5 for every
    electron (measured max 2.2e-5, median 1e-5).  The velocity bound is
    that of FP32 state, not of the orbits: at omega_c dt = 1.76 rad per step
    each component passes through about ten roundings at the scale of |v| per
    step (Boris rotation, both half accelerations, the r map), a random walk
    of ~3e-8 x sqrt(10 x 1000); the FP64 oracle itself carries a 6e-8
    perturbation of its inputs to only 1e-7 over the same run."""
    from cases import penning_rz

    g, o, _ = _trajectory_case(m, tmp_path, penning_rz, 1000, 2000, 0)
    _, ep, dvv, _ = _trajectory_errors(g, o, 5e-3, 20e-3)
    assert ep.max() <= 1e-5, ep.max()
    assert dvv.max() <= 5e-5, (dvv.max(), np.median(dvv))


def test_multipole_trajectories_1000_steps(m, tmp_path):
    """22-pole RF trap on the 257 x 257 grid of the bench workload, 2000 ions,
    1000 steps, collisions off: every position within 1e-5 of the domain size
    (measured max 2.8e-6).  Velocities: every ion whose orbit stays inside
    r < 0.7 r0 = 3.5 mm (the oracle's orbit) within |dv| <= 1e-5 v_rms
    (measured max 4e-6); every ion within 1e-4 v_rms (measured max 4.6e-5).
    The outer ions reach the RF wall, where the field grows as r^10 and turns
    a position difference into a velocity difference about ten times larger:
    the FP64 oracle itself carries a 6e-8 perturbation of its inputs to
    4e-6 v_rms on those ions (5e-7 on the inner ones), and the GPU's FP32
    rounding enters at every step."""
    from cases import multipole_xy

    g, o, rmax = _trajectory_case(m, tmp_path, multipole_xy, 1000, 2000, 1, track_r=(5e-3, 5e-3), collisions=False,
                                  n_nodes=257)
    common, ep, _, dvr = _trajectory_errors(g, o, 10e-3, 10e-3)
    assert ep.max() <= 1e-5, ep.max()
    inner = rmax[common] < 3.5e-3
    assert inner.sum() > 300
    assert dvr[inner].max() <= 1e-5, dvr[inner].max()
    assert dvr.max() <= 1e-4, dvr.max()


@pytest.mark.parametrize("direct", [-1, 1], ids=["multigrid", "inverse"])
def test_u_smooth_matches_oracle(m, tmp_path, direct):
    """u_smooth = 1 (Fields::u_smooth after each self-consistent solve): the
    GPU smoothing of the GPU potential equals the oracle's smoothing of the
    same potential bit for bit (last-column wrap and all), and the smoothed
    potential agrees with the oracle run's within 1e-7 relative: the GPU
    deposits positions quantised to 2^-20 cell, the oracle the FP64 ones
    (the solve itself is held to 1e-9 on a common rho above)."""
    from cases import penning_rz
    from mag2d_cases import load_port

    us = {}
    for sm in (0, 1):
        d = tmp_path / f"s{sm}"
        d.mkdir()
        cfg, species, inter, cpath, spath, parts = penning_rz(d, n=3000, mpf=2e4, u_smooth=sm)
        pic = m.Pic(cpath, spath, seed=3, direct_solve=direct)
        pic.speclist[0].set_particles(*parts)
        pic.advance_init()
        us[sm] = pic.field.u.copy()
        pic.close()
    L = load_port()
    want = np.zeros_like(us[0])
    L.orc_u_smooth(us[0].shape[0], us[0].shape[1], np.ascontiguousarray(us[0]).ctypes.data, want.ctypes.data)
    assert np.array_equal(us[1], want)
    assert np.abs(us[1] - us[0]).max() > 0.1  # the smoothing does act (it also reaches the electrodes)
    port = _port_for(m, cfg, species, inter, cpath, seed=3)
    port.set_particles(0, *parts)
    port.advance_init()
    ref = port.field(0)
    assert np.abs(us[1] - ref).max() <= 1e-7 * np.abs(ref).max()


def test_u_smooth_trajectories_500_steps(m, tmp_path):
    """A self-consistent Penning run with u_smooth = 1 against the oracle, 500
    steps: positions within 1e-5 of the domain size, velocities within the
    FP32 bound of the Penning test."""
    from cases import penning_rz

    g, o, _ = _trajectory_case(m, tmp_path, penning_rz, 500, 2000, 0, u_smooth=1)
    _, ep, dvv, _ = _trajectory_errors(g, o, 5e-3, 20e-3)
    assert ep.max() <= 1e-5, ep.max()
    assert dvv.max() <= 5e-5, dvv.max()


# ---------------------------------------------------------------------------
def _ks_2samp(a, b):
    a, b = np.sort(a), np.sort(b)
    allv = np.concatenate([a, b])
    cdf_a = np.searchsorted(a, allv, side="right") / len(a)
    cdf_b = np.searchsorted(b, allv, side="right") / len(b)
    d = np.abs(cdf_a - cdf_b).max()
    ne = len(a) * len(b) / (len(a) + len(b))
    lam = (math.sqrt(ne) + 0.12 + 0.11 / math.sqrt(ne)) * d
    p = 2 * sum((-1) ** (k - 1) * math.exp(-2 * k * k * lam * lam) for k in range(1, 101))
    return d, min(max(p, 0.0), 1.0)


def test_mcc_statistics_multipole(m, tmp_path):
    """Collision counts within 3 sigma and energy distributions alike (KS p > 0.01)."""
    from cases import multipole_xy
    from mag2d_cases import AMU, QE

    n, steps = 20_000, 200
    cfg, species, inter, cpath, spath, parts, loaded = multipole_xy(tmp_path, n=n, n_nodes=129, pressure=5.0)
    pic = m.Pic(cpath, spath, seed=11)
    ion = pic.speclist[1]
    ion.set_particles(*parts)
    pic.advance_init()
    pic.advance(steps)
    d = ion.diag()
    g = ion.particles()
    port = _port_for(m, cfg, species, inter, cpath, seed=11, loaded=loaded)
    port.set_particles(1, *parts)
    port.advance_init()
    port.advance(steps)
    o = port.particles(1)
    info = ion.info()
    prob = 1.0 - math.exp(-info["dt"] / info["lifetime"])
    # candidate count ~ Binomial(live * steps, prob); live changes little in this run
    live_mean = 0.5 * (n + d["n_live"])
    expect = live_mean * steps * prob
    cand = d["collisions"] + d["null_collisions"]
    assert abs(cand - expect) < 3 * math.sqrt(expect) + 0.01 * expect, (cand, expect)
    ncoll_oracle = port.collisions(1)
    assert abs(cand - ncoll_oracle) < 3 * math.sqrt(2 * expect), (cand, ncoll_oracle)
    eg = 0.5 * 3 * AMU * (g["vx"] ** 2 + g["vy"] ** 2 + g["vz"] ** 2) / QE
    lo = o[o[:, 7] == 0]
    eo = 0.5 * 3 * AMU * (lo[:, 3] ** 2 + lo[:, 4] ** 2 + lo[:, 5] ** 2) / QE
    _, p = _ks_2samp(eg, eo)
    assert p > 0.01, p
    pic.close()


def test_sort_does_not_change_results(m, tmp_path):
    """Random streams are keyed by particle id and the deposit is an integer sum,
    so sorting by cell every step or never gives bit-identical particles."""
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=5000)
    out, descents = [], []
    for si in (1, -1):
        pic = m.Pic(cpath, spath, seed=5, sort_interval=si)
        pic.speclist[0].set_particles(*parts)
        pic.advance_init()
        pic.advance(200)
        g = pic.speclist[0].particles()
        # slot order: cell index (r-major) of each live particle
        nz = pic.shape[1]
        cell = np.floor((g["x"] - pic.x_min) / pic.dx).astype(np.int64) * (nz - 1) + \
            np.floor((g["z"] - pic.z_min) / pic.dz).astype(np.int64)
        descents.append(np.mean(np.diff(cell) < 0))
        order = np.argsort(g["id"])
        out.append({k: v[order] for k, v in g.items()})
        pic.close()
    for k in ("id", "x", "z", "vx", "vy", "vz"):
        assert np.array_equal(out[0][k], out[1][k]), k
    # sorted one step ago: only particles that crossed a cell edge since are out of order
    assert descents[0] < 0.2 and descents[1] > 0.3, descents


def test_scrambled_sort_three_passes(m, tmp_path):
    """5e6 particles loaded in random order take the three-pass sort (blocks of
    cells, smaller blocks, cells): the particles after 3 steps are bit-identical
    to a run that never sorts, and they sit in cell order."""
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=5_000_000, nr=257, nz=513)
    out, descents = [], []
    for si in (1, -1):
        pic = m.Pic(cpath, spath, seed=8, sort_interval=si)
        pic.speclist[0].set_particles(*parts)
        pic.advance_init()
        pic.advance(3)
        g = pic.speclist[0].particles()
        nz = pic.shape[1]
        cell = np.floor((g["x"] - pic.x_min) / pic.dx).astype(np.int64) * (nz - 1) + \
            np.floor((g["z"] - pic.z_min) / pic.dz).astype(np.int64)
        descents.append(np.mean(np.diff(cell) < 0))
        order = np.argsort(g["id"])
        out.append({k: v[order] for k, v in g.items()})
        pic.close()
    assert len(out[0]["id"]) > 4_000_000
    for k in ("id", "x", "z", "vx", "vy", "vz"):
        assert np.array_equal(out[0][k], out[1][k]), k
    assert descents[0] < 0.2 and descents[1] > 0.3, descents


def test_inverse_solve_partial_rows_cover_the_particles(m, tmp_path):
    """A step's direct solve computes only the nodes within two of a charged
    node; reading u (which completes it) every step must not change a single
    particle: every face the particles read comes from computed nodes."""
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=20000)
    out = []
    for read_every_step in (False, True):
        pic = m.Pic(cpath, spath, seed=4, direct_solve=1)
        pic.speclist[0].set_particles(*parts)
        pic.advance_init()
        for _ in range(40):
            pic.advance(1)
            if read_every_step:
                _ = pic.field.u
        g = pic.speclist[0].particles()
        order = np.argsort(g["id"])
        out.append(({k: v[order] for k, v in g.items()}, pic.field.u))
        pic.close()
    for k in ("id", "x", "z", "vx", "vy", "vz"):
        assert np.array_equal(out[0][0][k], out[1][0][k]), k
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("case", ["multipole_rf_mcc", "penning_external"])
@pytest.mark.parametrize("fused", [64, 7])
def test_fused_steps_bit_identical(m, tmp_path, case, fused):
    """Where particles do not interact (no self-consistent field, background
    collision targets) several steps run as one launch per species.  The
    particles, counters and step counters equal those of the same steps run
    one launch at a time: 22-pole RF field with elastic collisions on a dense
    background (about 8000 collisions), and the Penning r-z field of the
    electrodes alone with B (cylindrical mover)."""
    from cases import multipole_xy, penning_rz

    if case == "multipole_rf_mcc":
        cfg, species, inter, cpath, spath, parts, _ = multipole_xy(tmp_path, n=20000, n_nodes=65, pressure=10.0)
        sp = 1
    else:
        cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=20000, selfconsistent=0)
        sp = 0
    out = []
    for mf in (1, fused):
        pic = m.Pic(cpath, spath, seed=9, sort_interval=20, max_fused_steps=mf)
        ion = pic.speclist[sp]
        ion.set_particles(*parts)
        pic.advance_init()
        pic.advance(3)
        pic.advance(150)
        g = ion.particles()
        order = np.argsort(g["id"])
        d = ion.diag()
        out.append(({k: v[order] for k, v in g.items()}, d))
        pic.close()
    (a, da), (b, db) = out
    for k in ("id", "x", "z", "vx", "vy", "vz"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("n_live", "collisions", "null_collisions", "removed", "particle_steps", "niter"):
        assert da[k] == db[k], (k, da[k], db[k])
    if case == "multipole_rf_mcc":
        assert da["collisions"] > 1000, da


@pytest.mark.parametrize("n", [20_000, 200_000], ids=["500_per_step", "5000_per_step"])
def test_mcc_candidate_list_path(m, tmp_path, n):
    """Charge exchange with a neutral background and Coulomb collisions with a
    second ion species that holds particles (partner = random live particle):
    collision counts against the oracle within 3 sigma, with about 500 and
    about 5000 candidates per step."""
    from mag2d_cases import AMU, QE, write_config, write_species_conf

    cfg = dict(coord="CARTESIAN", boundary="PERIODIC", geometry="EMPTY", x_max=1e-2, z_max=1e-2, x_sampl=9,
               z_sampl=9, selfconsistent=0, rf=0, extern_field=50.0, do_plot=0)
    sp = [dict(name="AR", type="NEUTRAL", mass=40 * AMU, density=5e21, temperature=300.0),
          dict(name="ARP", type="ION", mass=40 * AMU, charge=QE, dt=1e-8, density=1e16, temperature=3000.0,
               emax=5.0),
          dict(name="HEP", type="ION", mass=4 * AMU, charge=QE, dt=1e-8, density=1e16, temperature=3000.0,
               emax=5.0)]
    inter = [dict(name="cx", type="CX", primary="ARP", secondary="AR", rate=5e-16),
             dict(name="coul", type="COULOMB", primary="ARP", secondary="HEP"),
             dict(name="hel", type="ELASTIC", primary="HEP", secondary="AR", rate=3e-16)]
    cpath = write_config(cfg, tmp_path / "c.txt")
    spath = write_species_conf(sp, inter, tmp_path / "s.txt")
    rng = np.random.default_rng(4)
    steps = 50
    vth = np.sqrt(1.380662e-23 * 3000.0 / (40 * AMU))
    def parts(mass):
        v = np.sqrt(1.380662e-23 * 3000.0 / mass)
        return (1e-2 * rng.random(n), 1e-2 * rng.random(n), v * rng.standard_normal(n), v * rng.standard_normal(n),
                v * rng.standard_normal(n))
    pa, ph = parts(40 * AMU), parts(4 * AMU)
    pic = m.Pic(cpath, spath, seed=9)
    pic.speclist[1].set_particles(*pa)
    pic.speclist[2].set_particles(*ph)
    pic.advance_init()
    pic.advance(steps)
    d1, d2 = pic.speclist[1].diag(), pic.speclist[2].diag()
    port = _port_for(m, cfg, sp, inter, cpath, seed=9)
    port.set_particles(1, *pa)
    port.set_particles(2, *ph)
    port.advance_init()
    port.advance(steps)
    for s, d in ((1, d1), (2, d2)):
        cand = d["collisions"] + d["null_collisions"]
        ref = port.collisions(s)
        assert ref > 100
        assert abs(cand - ref) < 3 * math.sqrt(2 * ref), (s, cand, ref)
    pic.close()


@pytest.mark.parametrize("case", ["multipole_mcc", "penning_b"])
def test_push_variants_bit_identical(m, tmp_path, case):
    """The particle kernel's slots-per-thread variants (1, 2, 4) run the same
    per-particle arithmetic and the same keyed random streams: identical
    particles, counters and charge after 100 steps, with collisions (22-pole
    trap) and with a magnetic field and self-consistent deposit (Penning)."""
    from cases import multipole_xy, penning_rz

    combos = [1, 2, 4]
    out = []
    for vec in combos:
        if case == "multipole_mcc":
            cfg, species, inter, cpath, spath, parts, loaded = multipole_xy(tmp_path, n=10_001, n_nodes=129,
                                                                            pressure=5.0)
            pic = m.Pic(cpath, spath, seed=3, push_vec=vec)
            sp = pic.speclist[1]
        else:
            cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=10_001)
            pic = m.Pic(cpath, spath, seed=3, push_vec=vec)
            sp = pic.speclist[0]
        sp.set_particles(*parts)
        pic.advance_init()
        pic.advance(100)
        g = sp.particles()
        d = sp.diag()
        order = np.argsort(g["id"])
        out.append(({k: v[order] for k, v in g.items()}, d, sp.rho_fixed() if case == "penning_b" else None))
        pic.close()
    if case == "multipole_mcc":
        assert out[0][1]["collisions"] > 50
    for vec, (g, d, r) in zip(combos[1:], out[1:]):
        for k in ("id", "x", "z", "vx", "vy", "vz"):
            assert np.array_equal(g[k], out[0][0][k]), (vec, k)
        for k in ("n_live", "collisions", "null_collisions", "removed", "particle_steps"):
            assert d[k] == out[0][1][k], (vec, k)
        if r is not None:
            assert np.array_equal(r, out[0][2])


def test_multicoll_mover_statistics(m, tmp_path):
    """ADVANCE_MULTICOLL (event-driven free flight to each collision, FP64 time
    to the next collision): the number of scatter events within 3 sigma of the
    oracle's and the energy distributions alike (KS p > 0.01), electrons in He
    with the reference's cross-section tables in a 1000 V/m field."""
    import json

    from mag2d_cases import write_config, write_species_conf

    d = np.load(Path(__file__).resolve().parent / "golden" / "step_multicoll_eedf.npz")
    meta = json.loads(str(d["meta"]))
    cfg, sp, inter = meta["cfg"], meta["species"], meta["inter"]
    cpath = write_config(cfg, tmp_path / "c.txt")
    spath = write_species_conf(sp, inter, tmp_path / "s.txt")
    n, steps = 20000, 60
    ini = tmp_path / "init.txt"
    ini.write_text(f"add_particles_everywhere ELECTRON {n}\n")
    pic = m.Pic(cpath, spath, ini, seed=4)
    pic.advance_init()
    pic.advance(steps)
    g = pic.speclist[1].particles()
    dg = pic.speclist[1].diag()
    port = _port_for(m, cfg, sp, inter, cpath, seed=4)
    port.run_initscript(ini)
    port.advance_init()
    port.advance(steps)
    o = port.particles(1)
    events = dg["collisions"] + dg["null_collisions"]
    ref = port.collisions(1)
    assert ref > 1000
    assert abs(events - ref) < 3 * math.sqrt(2 * ref), (events, ref)
    me = 9.11e-31
    eg = 0.5 * me * (g["vx"] ** 2 + g["vy"] ** 2 + g["vz"] ** 2) / 1.602189e-19
    lo = o[o[:, 7] == 0]
    eo = 0.5 * me * (lo[:, 3] ** 2 + lo[:, 4] ** 2 + lo[:, 5] ** 2) / 1.602189e-19
    _, p = _ks_2samp(eg, eo)
    assert p > 0.01, (p, eg.mean(), eo.mean())
    pic.close()
