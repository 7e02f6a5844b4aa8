"""The C++ time-loop driver plasma2d_gpu (the reference's src/test.cpp:18-97 on
the C ABI) run end to end on a reference-style config / species_conf /
initscript triple.

The files it writes are checked two ways:
  * against the same run made through the Python binding of the same C ABI
    (same seed, same chunks of t_print steps): the live counts of out.dat and
    <species>.dat equal, the mean energies and potential.dat equal to the
    precision the driver prints (6 significant digits);
  * against the oracle running the same triple (the reference's algorithm with
    its own random numbers): live counts within 3 sigma of the oracle's, mean
    energies within 3 standard errors.
"""
from __future__ import annotations

import json
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
DRIVER = Path(__file__).resolve().parents[1] / "mag2d_gb300" / "lib" / "plasma2d_gpu"


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def _read_rows(path):
    return np.array([[float(x) for x in line.split()] for line in Path(path).read_text().splitlines() if line.strip()])


def test_driver_end_to_end(m, tmp_path):
    from mag2d_cases import Port, write_config, write_species_conf

    meta = json.loads(str(np.load(GOLDEN / "step_rf22_mcc.npz")["meta"]))
    niter, t_print = 200, 50
    cfg = dict(meta["cfg"], niter=niter, t_print=t_print)
    species, inter = meta["species"], meta["inter"]
    cpath = write_config(cfg, tmp_path / "config.txt")
    spath = write_species_conf(species, inter, tmp_path / "species_conf.txt")
    ini = tmp_path / "initscript.txt"
    ini.write_text("add_particles_on_disk IONS 8000 1e-2 1e-2 3e-3\nadd_particles_everywhere IONS 4000\n"
                   "add_particles_bessel IONS 8000 1e-2 1e-2 2e-3\n")
    out = tmp_path / "output"
    r = subprocess.run([str(DRIVER), f"config={cpath}", f"species_conf={spath}", f"initscript={ini}",
                        f"output_dir={out}", "seed=7"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    od = _read_rows(out / "out.dat")
    ions = _read_rows(out / "IONS.dat")
    pot = _read_rows(out / "potential.dat")
    assert od.shape == (niter // t_print, 2 + len(species))
    assert np.array_equal(od[:, 0], np.arange(t_print, niter + 1, t_print))
    assert np.array_equal(ions[:, 0], od[:, 0])
    assert np.allclose(ions[:, 3], ions[:, 0] * species[1]["dt"], rtol=1e-5)

    # the same run through the Python binding
    pic = m.Pic(cpath, spath, ini, seed=7)
    pic.advance_init()
    api = []
    for _ in range(niter // t_print):
        pic.advance(t_print)
        d = pic.speclist[1].diag()
        api.append((d["n_live"], d["mean_energy_eV"]))
    u = pic.field.u
    x0, z0, dx, dz = pic.x_min, pic.z_min, pic.dx, pic.dz
    pic.close()
    api = np.array(api)
    assert np.array_equal(od[:, 3], api[:, 0]) and np.array_equal(ions[:, 1], api[:, 0])
    assert np.allclose(ions[:, 2], api[:, 1], rtol=1e-5, atol=0)
    nx, nz = u.shape
    assert pot.shape == (nx * nz, 3)
    assert np.allclose(pot[:, 0], np.repeat(x0 + dx * np.arange(nx), nz), rtol=1e-5, atol=1e-12)
    assert np.allclose(pot[:, 1], np.tile(z0 + dz * np.arange(nz), nx), rtol=1e-5, atol=1e-12)
    assert np.allclose(pot[:, 2], u.reshape(-1), rtol=1e-5, atol=1e-5 * max(np.abs(u).max(), 1e-30))

    # the oracle on the same triple (its own loaders and random numbers)
    mask, volt = m.config_geometry(cpath)
    port = Port(cfg, species, inter, mask, volt, seed=7)
    port.run_initscript(ini)
    port.advance_init()
    n_start = port.n_live(1)
    mion = species[1]["mass"]
    for k in range(niter // t_print):
        port.advance(t_print)
        o = port.particles(1)
        live = o[o[:, 7] == 0]
        e = 0.5 * mion * (live[:, 3] ** 2 + live[:, 4] ** 2 + live[:, 5] ** 2) / 1.602189e-19
        # live counts: the loaders keep a binomial share of their draws inside the
        # domain and the run loses a binomial share at the boundary
        sig = math.sqrt(n_start * 0.25 + len(live) * 0.25)
        assert abs(api[k, 0] - len(live)) <= 3 * sig, (k, api[k, 0], len(live))
        se = e.std() / math.sqrt(len(e))
        assert abs(api[k, 1] - e.mean()) <= 3 * math.sqrt(2) * se, (k, api[k, 1], e.mean(), se)
