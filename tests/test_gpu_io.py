"""Particle files (BaseSpecies::save / load, particle_reload) through the GPU state."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def test_save_load_round_trip(m, tmp_path):
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=5000)
    a = m.Pic(cpath, spath, seed=2)
    a.speclist[0].set_particles(*parts)
    a.advance_init()
    a.advance(20)
    a.speclist[0].save(tmp_path / "e.dat")
    ga = a.speclist[0].particles()
    f = m.read_particle_file(tmp_path / "e.dat")
    assert len(f["x"]) == len(ga["x"])
    b = m.Pic(cpath, spath, seed=2)
    b.speclist[0].load(tmp_path / "e.dat")
    gb = b.speclist[0].particles()
    for k in ("x", "z", "vx", "vy", "vz"):
        assert np.array_equal(ga[k], gb[k]), k
    a.close()
    b.close()


def test_load_redraws_particles_outside_the_domain(m, tmp_path):
    """As BaseSpecies::load: particles inside the domain load unchanged, those
    outside are redrawn uniformly inside it (the reference's own result on the
    same file is the golden fixture)."""
    from mag2d_cases import QE, write_config, write_species_conf
    import json

    d = np.load(GOLDEN / "particles.npz")
    cfg = json.loads(str(d["meta"]))["cfg"]
    cp = write_config(cfg, tmp_path / "c.txt")
    sp = write_species_conf([dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11,
                                  temperature=11604.5)], [], tmp_path / "s.txt")
    m.write_particle_file(tmp_path / "oob.dat", d["x_oob"], d["z_oob"], d["vx"], d["vy"], d["vz"])
    pic = m.Pic(cp, sp, seed=3)
    pic.speclist[0].load(tmp_path / "oob.dat")
    g = pic.speclist[0].particles()
    order = np.argsort(g["id"])
    x, z = g["x"][order], g["z"][order]
    ref = d["loaded"]
    inside = (d["x_oob"] >= 0) & (d["x_oob"] <= 1e-2) & (d["z_oob"] >= 0) & (d["z_oob"] <= 2e-2)
    assert (~inside).sum() == 3
    assert np.abs(x[inside] - ref[inside, 0]).max() <= 1e-2 * 2.0 ** -20
    assert np.abs(z[inside] - ref[inside, 2]).max() <= 2e-2 * 2.0 ** -20
    assert ((x >= 0) & (x <= 1e-2) & (z >= 0) & (z <= 2e-2)).all()
    assert np.array_equal(g["vz"][order], d["vz"].astype(np.float32))
    pic.close()


def test_particle_reload_at_creation(m, tmp_path):
    """particle_reload = 1 loads every species from particle_reload_dir when the
    simulation is made (src/pic.cpp:138-146)."""
    from cases import penning_rz
    from mag2d_cases import write_config

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=3000)
    a = m.Pic(cpath, spath, seed=2)
    a.speclist[0].set_particles(*parts)
    rd = tmp_path / "reload"
    rd.mkdir()
    a.speclist[0].save(rd / "particles_ELECTRON.dat")
    cfg2 = dict(cfg, particle_reload=1, particle_reload_dir=str(rd))
    c2 = write_config(cfg2, tmp_path / "reload.txt")
    b = m.Pic(c2, spath, seed=2)
    assert b.speclist[0].diag()["n_live"] == a.speclist[0].diag()["n_live"] == 3000
    with pytest.raises(Exception):
        m.Pic(write_config(dict(cfg, particle_reload=1, particle_reload_dir=str(tmp_path / "none")),
                           tmp_path / "r2.txt"), spath)
    a.close()
    b.close()


def test_sampled_distributions(m, tmp_path):
    """dist_sample on the GPU: the energy histogram equals Histogram::add of the
    particles' energies (the reference's formula in FP64 on the same FP32
    velocities), rhoAverage of one sample is the charge deposit, uAvg the
    potential; print_distribution writes the reference's file layouts."""
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=20000)
    pic = m.Pic(cpath, spath, seed=2)
    e = pic.speclist[0]
    e.set_particles(*parts)
    pic.advance_init()
    pic.advance(10)
    pic.dist_reset()
    pic.dist_sample()
    g = e.particles()
    info = e.info()
    mass, emax = info["mass"], info["E_max"]
    vx, vy, vz = (np.asarray(g[k], dtype=np.float32).astype(np.float64) for k in ("vx", "vy", "vz"))
    f = (vx * vx + vz * vz + vy * vy) * mass * 0.5 / 1.602189e-19
    inside = (f < emax) & (f > 0.0)
    bins = np.zeros(200)
    np.add.at(bins, np.minimum((f[inside] * 200 / emax).astype(int), 199), 1)
    d = e.energy_dist()
    norm = inside.sum() * emax / 200
    assert d["n_val"] == inside.sum() and d["n_val_tot"] == len(f)
    assert np.abs(d["values"] * norm - bins).sum() <= 4  # bin-edge ties from FMA contraction at most
    assert abs(d["mean_tot"] - f.mean()) <= 1e-12 * f.mean()
    q = info["charge"] * 2.0 ** -40
    assert np.allclose(e.rho_average, e.rho_fixed() * q, rtol=1e-15, atol=0)
    u1 = pic.field.u
    assert np.array_equal(pic.u_average, u1)
    pic.advance(5)
    pic.dist_sample()
    u2 = pic.field.u
    assert np.allclose(pic.u_average, 0.5 * (u1 + u2), rtol=1e-14, atol=1e-14 * np.abs(u1).max())
    pic.print_distribution(tmp_path)
    pic.print_field(tmp_path / "potential.dat")
    lines = (tmp_path / "ELECTRON_energy_dist.dat").read_text().splitlines()
    assert len(lines) == 200 and len(lines[0].split("\t")) == 2
    rho_lines = (tmp_path / "ELECTRON_rho.dat").read_text().split("\n")
    nx, nz = pic.shape
    assert sum(1 for line in rho_lines if line.count("\t") == 2) == nx * nz
    pic.close()


@pytest.mark.parametrize("selfconsistent", [0, 1])
def test_set_electrode_voltages_matches_a_fresh_run(m, tmp_path, selfconsistent):
    """mag_set_electrode_voltages: the fields of the new voltages equal those of
    a run made from a config with them (within the solver tolerance)."""
    from cases import penning_rz
    from mag2d_cases import write_config

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=3000, selfconsistent=selfconsistent)
    cfg2 = dict(cfg, u_endcap=-17.5)
    cpath2 = write_config(cfg2, tmp_path / "c2.txt")
    b = m.Pic(cpath2, spath, seed=2)
    v_new = b.field.voltage
    a = m.Pic(cpath, spath, seed=2)
    a.set_electrode_voltages(v_new)
    for p in (a, b):
        p.speclist[0].set_particles(*parts)
        p.advance_init()
        p.advance(5)
    ua, ub = a.field.u, b.field.u
    assert np.abs(ua - ub).max() <= 1e-9 * np.abs(ub).max()
    ga, gb = a.speclist[0].particles(), b.speclist[0].particles()
    oa, ob = np.argsort(ga["id"]), np.argsort(gb["id"])
    assert np.array_equal(ga["id"][oa], gb["id"][ob])
    assert np.abs(ga["z"][oa] - gb["z"][ob]).max() <= 1e-9 * 20e-3
    a.close()
    b.close()


def test_n_live_and_aos_records(m, tmp_path):
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=4000)
    pic = m.Pic(cpath, spath, seed=2)
    sp = pic.speclist[0]
    sp.set_particles(*parts)
    pic.advance_init()
    pic.advance(30)
    g = sp.particles()
    rec = sp.particles_aos()
    assert sp.n_live() == sp.diag()["n_live"] == len(g["x"]) == len(rec)
    for c, k in ((0, "x"), (2, "z"), (3, "vx"), (4, "vy"), (5, "vz")):
        assert np.array_equal(rec[:, c], g[k]), k
    assert np.all(rec[:, 1] == 0) and np.all(rec[:, 7] == 0)
    pic.close()


def test_set_particles_from_page_locked_memory(m, tmp_path):
    """Page-locked host arrays are read in place by the conversion kernel,
    other arrays through a device staging copy: both give the same state, and
    the diagnostics (one reduction, one synchronisation) agree with the
    particles read back."""
    torch = pytest.importorskip("torch")
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=30000)
    # a few particles outside the box are removed on the way in
    parts = [np.array(a) for a in parts]
    parts[0][:7] = 1.0
    pinned = []
    for a in parts:
        buf = torch.empty(len(a), dtype=torch.float64).pin_memory()
        buf.numpy()[:] = a
        pinned.append(buf)
    out = []
    for src in (parts, [b.numpy() for b in pinned]):
        pic = m.Pic(cpath, spath, seed=2)
        sp = pic.speclist[0]
        sp.set_particles(*src)
        g = sp.particles()
        d = sp.diag()
        assert d["n_live"] == len(g["x"]) == 30000 - 7
        e = 0.5 * 9.11e-31 * np.mean(g["vx"] ** 2 + g["vy"] ** 2 + g["vz"] ** 2) / 1.602189e-19
        assert abs(d["mean_energy_eV"] - e) <= 1e-6 * e
        out.append(g)
        pic.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


def test_print_trace_of_tracked_particles(m, tmp_path):
    """Pic::print_trace: a particle added by add_tracked_particle gets one
    "x z vx vz vy" line per call in <species>_traj_<slot>.dat, equal to its
    state read back through the particle view."""
    from mag2d_cases import QE, write_config, write_species_conf

    cfg = dict(coord="CARTESIAN", boundary="PERIODIC", geometry="EMPTY", x_max=2e-2, z_max=2e-2, x_sampl=11,
               z_sampl=11, selfconsistent=0, rf=0, extern_field=100.0, do_plot=0)
    sp = [dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, density=1e15,
               temperature=11604.5)]
    cpath = write_config(cfg, tmp_path / "c.txt")
    spath = write_species_conf(sp, [], tmp_path / "s.txt")
    ini = tmp_path / "init.txt"
    ini.write_text("add_particles_everywhere ELECTRON 500\nadd_tracked_particle ELECTRON 1e-2 1e-2 1000 2000 3000\n")
    out = tmp_path / "out"
    out.mkdir()
    pic = m.Pic(cpath, spath, ini, seed=1)
    pic.advance_init()
    for _ in range(3):
        pic.advance(10)
        pic.print_trace(out)
    lines = (out / "ELECTRON_traj_500.dat").read_text().splitlines()
    assert len(lines) == 3
    last = np.array([float(v) for v in lines[-1].split()])
    g = pic.speclist[0].particles()
    k = int(np.flatnonzero(g["id"] == 500)[0])
    want = np.array([g["x"][k], g["z"][k], g["vx"][k], g["vz"][k], g["vy"][k]])
    assert np.allclose(last, want, rtol=1e-9, atol=0), (last, want)
    pic.close()
