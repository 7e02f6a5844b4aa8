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
