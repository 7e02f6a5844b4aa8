"""Particle source (use_source; Species<CARTESIAN>::source5_refresh / source,
src/particles.cpp:1052-1226) on the GPU, against the reference's own run
(tests/golden/source.npz and its source5_save file, made by make_golden.py).

The box particles are drawn from other random streams than the reference's,
so the comparisons are statistical: the domain fills through its faces at the
reference's rate (live counts within 5 % + 4 sigma every 10 steps), and the
copies a box makes equal the face crossings its own velocities imply."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def _read_box(path):
    """source5 file: int32 count, then 64-byte records (7 doubles, bool, padding)."""
    raw = Path(path).read_bytes()
    n = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    rec = np.frombuffer(raw[4:4 + 64 * n], dtype=np.float64).reshape(n, 8)
    return n, rec[:, :7]


def _case(tmp_path):
    from mag2d_cases import write_config, write_species_conf

    g = np.load(GOLDEN / "source.npz", allow_pickle=True)
    meta = json.loads(str(g["meta"]))
    cpath = write_config(meta["cfg"], tmp_path / "src_cfg.txt")
    spath = write_species_conf(meta["species"], [], tmp_path / "src_sp.txt")
    return meta, cpath, spath, g


def _start(m, cpath, spath, seed=3):
    pic = m.Pic(cpath, spath, seed=seed)
    e = pic.speclist[0]
    e.set_particles(np.array([5e-3]), np.array([5e-3]), np.zeros(1), np.zeros(1), np.zeros(1))
    pic.advance_init()  # refreshes the source boxes with src_fact
    return pic, e


def test_source_box_file_round_trip_of_reference(m, tmp_path):
    """The reference's source5_save file loads into the box and saves back
    record for record (velocities rounded to the FP32 state)."""
    meta, cpath, spath, _ = _case(tmp_path)
    pic, e = _start(m, cpath, spath)
    info = e.source_info()
    assert info["n_box"] == int(meta["species"][0]["density"] * 1e5 / 1e13 / meta["cfg"]["src_fact"])
    e.source_load(GOLDEN / "source_ref.dat")
    e.source_save(tmp_path / "back.dat")
    n0, r0 = _read_box(GOLDEN / "source_ref.dat")
    n1, r1 = _read_box(tmp_path / "back.dat")
    assert n0 == n1 == e.source_info()["n_box"]
    assert np.array_equal(r0[:, 0], r1[:, 0]) and np.array_equal(r0[:, 2], r1[:, 2])
    for c in (3, 4, 5):
        assert np.array_equal(r0[:, c].astype(np.float32).astype(np.float64), r1[:, c])
    pic.close()


def test_source_inflow_matches_reference(m, tmp_path):
    meta, cpath, spath, g = _case(tmp_path)
    pic, e = _start(m, cpath, spath)
    e.source_save(tmp_path / "box0.dat")
    _, box = _read_box(tmp_path / "box0.dat")
    live = [e.diag()["n_live"]]
    for _ in range(30):
        pic.advance(10)
        live.append(e.diag()["n_live"])
    live = np.array(live)
    ref = g["live"]
    assert np.array_equal(g["steps"], np.arange(0, 301, 10))
    sel = g["steps"] >= 20
    tol = 0.05 * ref[sel] + 4 * np.sqrt(ref[sel])
    assert np.all(np.abs(live[sel] - ref[sel]) <= tol), (live, ref)
    # copies = face crossings of the periodic box: without collisions and
    # field, box particle i crosses |v_i| T dt / b times (+-1) in T steps
    cfg, sp = meta["cfg"], meta["species"][0]
    bx = cfg["x_max"] / cfg["src_fact"]
    bz = cfg["z_max"] / cfg["src_fact"]
    expect = (np.abs(box[:, 3]) / bx + np.abs(box[:, 5]) / bz).sum() * sp["dt"] * 300
    info = e.source_info()
    assert info["dropped"] == 0
    assert abs(info["injected"] - expect) <= 0.03 * expect, (info, expect)
    pic.close()


def test_source_deterministic(m, tmp_path):
    """Copies are appended in box order with ids from a scan, so two runs are
    identical particle for particle."""
    meta, cpath, spath, _ = _case(tmp_path)
    out = []
    for _ in range(2):
        pic, e = _start(m, cpath, spath, seed=11)
        pic.advance(60)
        g = e.particles()
        order = np.argsort(g["id"])  # the sort by cell does not keep slot order within a cell
        out.append({k: v[order] for k, v in g.items()})
        pic.close()
    for k in ("id", "x", "z", "vx", "vy", "vz"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_source_refused_where_the_reference_has_none(m, tmp_path):
    """Cylindrical runs: Species<CYLINDRICAL>::source is declared but not
    defined in the reference (particles.hpp:311)."""
    from cases import penning_rz
    from mag2d_cases import write_config

    cfg, species, inter, cpath, spath, parts = penning_rz(tmp_path, n=10)
    cfg = dict(cfg, use_source=1)
    cpath = write_config(cfg, tmp_path / "cyl_src.txt")
    with pytest.raises(Exception, match="source"):
        m.Pic(cpath, spath, seed=1)
