"""Edge cases of the step through the C ABI: empty species, every particle
leaving at once, particles on the far boundary (deposit bit-exact), empty
particle arrays, and grids beyond the fixed-point position range."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def test_empty_species_self_consistent_run(m, tmp_path):
    """No particles: the steps run, count nothing, and the potential is the
    electrodes' own (the same as a Poisson solve of zero charge)."""
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=10)
    pic = m.Pic(cpath, spath, seed=1)
    sp = pic.speclist[0]
    pic.advance_init()
    pic.advance(10)
    d = sp.diag()
    assert d["n_live"] == 0 and d["removed"] == 0 and d["particle_steps"] == 0
    u = pic.field.u.copy()
    pic.field.set_rho(np.zeros(pic.shape))
    pic.field.boundary_solve()
    assert np.abs(pic.field.u - u).max() <= 1e-9 * np.abs(u).max()
    pic.close()


def test_empty_particle_arrays(m, tmp_path):
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=10)
    pic = m.Pic(cpath, spath, seed=1)
    sp = pic.speclist[0]
    sp.set_particles(*[np.zeros(0) for _ in range(5)])
    pic.advance_init()
    pic.advance(3)
    assert sp.n_live() == 0
    assert len(sp.particles()["x"]) == 0
    pic.close()


def test_every_particle_leaves_in_one_step(m, tmp_path):
    """FREE boundary: particles moving out of the box in one step are all
    removed, counted, and the run continues with none."""
    from cases import penning_rz

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=5000)
    x, z, vx, vy, vz = (np.array(a) for a in parts)
    vz[:] = 1e10 * np.where(np.arange(len(vz)) % 2 == 0, 1.0, -1.0)  # 0.1 m per 10 ps step
    pic = m.Pic(cpath, spath, seed=1)
    sp = pic.speclist[0]
    sp.set_particles(x, z, vx, vy, vz)
    pic.advance_init()
    pic.advance(1)
    d = sp.diag()
    assert d["n_live"] == 0 and d["removed"] == 5000
    pic.advance(25)  # through a sort that compacts the removed slots
    d = sp.diag()
    assert d["n_live"] == 0 and d["removed"] == 5000
    assert np.all(sp.rho_fixed() == 0)
    pic.close()


def test_deposit_on_the_far_boundary_bit_exact(m, tmp_path):
    """Particles on the last node line (x = x_max, z = z_max) belong to the
    last cell with a full weight on its far corners, as in the oracle."""
    from cases import penning_rz
    from mag2d_cases import deposit_fixed, to_fixed

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=10)
    pic = m.Pic(cpath, spath, seed=1)
    sp = pic.speclist[0]
    nx, nz = pic.shape
    rng = np.random.default_rng(4)
    n = 3000
    x = rng.uniform(pic.x_min, pic.x_min + (nx - 1) * pic.dx, n)
    z = rng.uniform(pic.z_min, pic.z_min + (nz - 1) * pic.dz, n)
    x[:1000] = pic.x_min + (nx - 1) * pic.dx
    z[500:1500] = pic.z_min + (nz - 1) * pic.dz
    x[1500:1600] = pic.x_min
    z[1600:1700] = pic.z_min
    sp.set_particles(x, z, np.zeros(n), np.zeros(n), np.zeros(n))
    pic.deposit()
    got = sp.rho_fixed()
    g = sp.particles()
    xg = to_fixed((g["x"] - pic.x_min) / pic.dx)
    zg = to_fixed((g["z"] - pic.z_min) / pic.dz)
    assert len(xg) == n
    assert np.array_equal(got, deposit_fixed(nx, nz, xg, zg))
    assert got.sum() == n << 40
    pic.close()


@pytest.mark.parametrize("key", ["r_sampl", "z_sampl"])
def test_grid_beyond_the_fixed_point_range_is_refused(m, tmp_path, key):
    from cases import penning_rz
    from mag2d_cases import write_config

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=10)
    cfg = dict(cfg, **{key: 4097})
    cpath = write_config(cfg, tmp_path / "big.txt")
    from mag2d_gb300._lib import MagError

    with pytest.raises(MagError, match="4096"):
        m.Pic(cpath, spath, seed=1)
