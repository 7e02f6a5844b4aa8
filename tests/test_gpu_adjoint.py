"""Adjoint gradients (mag_adjoint_run) against central finite differences.

Loss after N steps of the segmented Penning trap: mean axial kinetic energy
[eV] plus lost fraction.  The adjoint of the collisionless step (push, gather,
deposit, Poisson) with checkpoints gives d loss / d u_segment_k and
d loss / d Bz in one run; central differences need two forward runs per
parameter.  Against the oracle's FP64 runs (h = 1e-3 V, 1e-4 T) the bar is
1e-3 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = [f"u_segment_{k}" for k in range(8)]


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def _loss(m, tmp_path, volts, Bz, n, steps, tag):
    from cases import penning_segments
    from mag2d_gb300.autograd import loss_from_state

    c = penning_segments(tmp_path, n=n, volts=volts, Bz=Bz, tag=tag)
    pic = m.Pic(c[3], c[4], c[5], seed=c[6])
    n0 = pic.speclist[0].diag()["n_live"]
    pic.advance_init()
    pic.advance(steps)
    val = loss_from_state(pic, n0=n0)
    pic.close()
    return val


def _oracle_loss(m, tmp_path, volts, Bz, parts, steps, tag):
    """The loss of the oracle (the reference's algorithm in FP64) from the same initial particles."""
    from cases import penning_segments
    from mag2d_cases import Port

    cfg, species, inter, cpath, spath, ipath, seed = penning_segments(tmp_path, n=len(parts[0]), volts=volts, Bz=Bz,
                                                                      tag=tag)
    mask, volt = m.config_geometry(cpath)
    port = Port(cfg, species, inter, mask, volt, seed=1)
    port.set_particles(0, *parts)
    port.advance_init()
    port.advance(steps)
    o = port.particles(0)
    live = o[o[:, 7] == 0]
    e = 0.5 * species[0]["mass"] * live[:, 5] ** 2 / 1.602189e-19
    return float(e.mean()) + (len(parts[0]) - len(live)) / len(parts[0])


def _adjoint(m, tmp_path, n, steps, volts, Bz, direct=0):
    from cases import penning_segments

    c = penning_segments(tmp_path, n=n, volts=volts, Bz=Bz, tag="adj")
    pic = m.Pic(c[3], c[4], c[5], seed=c[6], direct_solve=direct)
    g0 = pic.speclist[0].particles()
    parts = tuple(np.asarray(g0[k], dtype=np.float64) for k in ("x", "z", "vx", "vy", "vz"))
    info, grad = pic.adjoint(steps, KEYS, checkpoint=64, grad_b=True)
    pic.close()
    return info, grad, parts


@pytest.mark.parametrize("direct", [0, -1], ids=["inverse", "multigrid"])
def test_adjoint_matches_oracle_finite_differences(m, tmp_path, direct):
    """Central differences of the oracle (FP64, h = 1e-3 V and 1e-4 T) from the
    same initial particles: agreement within 1e-3 relative, with the forward
    and transposed solves by the precomputed inverse or by multigrid."""
    n, steps = 20_000, 300
    volts = np.random.default_rng(7).uniform(-15.0, -5.0, 8)
    Bz = 1.0
    info, grad, parts = _adjoint(m, tmp_path, n, steps, volts, Bz, direct)
    assert info["n_live"] > 0.9 * info["n0"], info
    scale = np.abs(grad[:8]).max()
    assert scale > 0
    for k in (2, 5):
        h = 1e-3
        vp, vm = volts.copy(), volts.copy()
        vp[k] += h
        vm[k] -= h
        fd = (_oracle_loss(m, tmp_path, vp, Bz, parts, steps, f"op{k}")
              - _oracle_loss(m, tmp_path, vm, Bz, parts, steps, f"om{k}")) / (2 * h)
        assert abs(grad[k] - fd) <= 1e-3 * max(abs(fd), 0.05 * scale), (k, grad[k], fd)
    hb = 1e-4
    fd = (_oracle_loss(m, tmp_path, volts, Bz + hb, parts, steps, "obp")
          - _oracle_loss(m, tmp_path, volts, Bz - hb, parts, steps, "obm")) / (2 * hb)
    assert abs(grad[8 + 2] - fd) <= 1e-3 * abs(fd) + 1e-6, (grad[8 + 2], fd)


def test_adjoint_matches_gpu_finite_differences(m, tmp_path):
    """Central differences of the GPU's own forward runs.  The FP32 state adds
    rounding noise of about 1e-8 relative to the loss, so the steps are 1e-2 V
    and 1e-3 T and the bar 5e-3 relative; the forward part of the adjoint run
    reproduces the plain run's loss."""
    n, steps = 20_000, 300
    volts = np.random.default_rng(7).uniform(-15.0, -5.0, 8)
    Bz = 1.0
    info, grad, _ = _adjoint(m, tmp_path, n, steps, volts, Bz)
    base = _loss(m, tmp_path, volts, Bz, n, steps, "base")
    assert abs(base - info["loss"]) <= 1e-9 * abs(base) + 1e-12, (base, info)
    scale = np.abs(grad[:8]).max()
    for k in (2, 5):
        h = 1e-2
        vp, vm = volts.copy(), volts.copy()
        vp[k] += h
        vm[k] -= h
        fd = (_loss(m, tmp_path, vp, Bz, n, steps, f"p{k}") - _loss(m, tmp_path, vm, Bz, n, steps, f"m{k}")) / (2 * h)
        assert abs(grad[k] - fd) <= 5e-3 * max(abs(fd), 0.05 * scale), (k, grad[k], fd)
    # the axial energy hardly depends on Bz (about 1e-6 eV/T here): the FP32
    # noise floor of this difference, 1e-8 eV / 2e-3 T, sets the absolute bar
    hb = 1e-3
    fd = (_loss(m, tmp_path, volts, Bz + hb, n, steps, "bp") - _loss(m, tmp_path, volts, Bz - hb, n, steps, "bm")) / (2 * hb)
    assert abs(grad[8 + 2] - fd) <= 5e-3 * abs(fd) + 5e-6, (grad[8 + 2], fd)


def test_autograd_function(m, tmp_path):
    torch = pytest.importorskip("torch")
    from cases import penning_segments
    from mag2d_gb300.autograd import TrapLoss

    def make(v, b):
        c = penning_segments(tmp_path, n=5000, volts=v, Bz=float(b[2]), tag="ag")
        return m.Pic(c[3], c[4], c[5], seed=c[6])

    v = torch.tensor(np.random.default_rng(3).uniform(-15, -5, 8), dtype=torch.float64, requires_grad=True)
    b = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64, requires_grad=True)
    loss = TrapLoss.apply(v, b, make, 100, KEYS, 50)
    loss.backward()
    assert v.grad is not None and b.grad is not None
    assert torch.isfinite(v.grad).all() and torch.isfinite(b.grad).all()
    assert float(v.grad.abs().max()) > 0


def _oracle_loss_worker(args):
    """One oracle run for the process pool: (volts, Bz, parts, steps, tag, root) -> (loss, lost)."""
    volts, Bz, parts, steps, tag, root = args
    import sys
    import tempfile
    from pathlib import Path

    sys.path.insert(0, str(Path(root) / "tests"))
    sys.path.insert(0, str(root))
    import mag2d_gb300 as m
    from cases import penning_segments
    from mag2d_cases import Port

    with tempfile.TemporaryDirectory() as d:
        cfg, species, inter, cpath, spath, ipath, seed = penning_segments(Path(d), n=len(parts[0]), volts=volts,
                                                                          Bz=Bz, tag=tag)
        mask, volt = m.config_geometry(cpath)
    port = Port(cfg, species, inter, mask, volt, seed=1)
    port.set_particles(0, *parts)
    port.advance_init()
    port.advance(steps)
    o = port.particles(0)
    live = o[o[:, 7] == 0]
    e = 0.5 * species[0]["mass"] * live[:, 5] ** 2 / 1.602189e-19
    lost = len(parts[0]) - len(live)
    return float(e.mean()) + lost / len(parts[0]), lost


def test_adjoint_full_configuration(m, tmp_path):
    """The adjoint configuration as specified: 1e5 electrons, 2000 steps,
    checkpoints every 100 steps, the gradient with respect to all 8 segment
    voltages and B.  Every parameter against central differences of the GPU's
    own forward runs (h = 1e-2 V, 1e-3 T; FP32 rounding noise of the loss sets
    the 5e-3 bar), and voltages 2 and 5 and Bz against central differences of
    the oracle's FP64 runs from the same initial particles (h = 1e-3 V,
    1e-4 T) within 1e-3 relative.

    The lost fraction of the loss is piecewise constant in the parameters: a
    particle is either lost or not, so its pathwise derivative is zero and the
    adjoint seeds only the energy term.  A difference quotient agrees with
    that only while no particle changes its fate between the two runs; the
    test asserts that the lost counts of every pair of runs are equal."""
    import multiprocessing as mp
    from pathlib import Path

    from cases import penning_segments
    from mag2d_gb300.autograd import loss_from_state

    n, steps = 100_000, 2000
    volts = np.random.default_rng(7).uniform(-15.0, -5.0, 8)
    Bz = 1.0
    c = penning_segments(tmp_path, n=n, volts=volts, Bz=Bz, tag="full")
    pic = m.Pic(c[3], c[4], c[5], seed=c[6])
    g0 = pic.speclist[0].particles()
    parts = tuple(np.asarray(g0[k], dtype=np.float64) for k in ("x", "z", "vx", "vy", "vz"))
    info, grad = pic.adjoint(steps, KEYS, checkpoint=100, grad_b=True)
    pic.close()
    assert len(grad) == 11 and np.all(np.isfinite(grad))
    assert info["n_live"] > 0.9 * info["n0"], info

    def gpu_loss(v, b, tag):
        cc = penning_segments(tmp_path, n=n, volts=v, Bz=b, tag=tag)
        p = m.Pic(cc[3], cc[4], cc[5], seed=cc[6])
        n0 = p.speclist[0].diag()["n_live"]
        p.advance_init()
        p.advance(steps)
        val = loss_from_state(p, n0=n0)
        lost = n0 - p.speclist[0].diag()["n_live"]
        p.close()
        return val, lost

    scale = np.abs(grad[:8]).max()
    assert scale > 0
    for k in range(8):
        h = 1e-2
        vp, vm = volts.copy(), volts.copy()
        vp[k] += h
        vm[k] -= h
        (lp, np_), (lm, nm) = gpu_loss(vp, Bz, f"gp{k}"), gpu_loss(vm, Bz, f"gm{k}")
        assert np_ == nm, (k, np_, nm)
        fd = (lp - lm) / (2 * h)
        assert abs(grad[k] - fd) <= 5e-3 * max(abs(fd), 0.05 * scale), (k, grad[k], fd)
    hb = 1e-3
    (lp, np_), (lm, nm) = gpu_loss(volts, Bz + hb, "gbp"), gpu_loss(volts, Bz - hb, "gbm")
    assert np_ == nm
    fd = (lp - lm) / (2 * hb)
    assert abs(grad[10] - fd) <= 5e-3 * abs(fd) + 5e-6, (grad[10], fd)

    root = str(Path(__file__).resolve().parents[1])
    jobs = []
    for k in (2, 5):
        vp, vm = volts.copy(), volts.copy()
        vp[k] += 1e-3
        vm[k] -= 1e-3
        jobs += [(vp, Bz, parts, steps, f"op{k}", root), (vm, Bz, parts, steps, f"om{k}", root)]
    jobs += [(volts, Bz + 1e-4, parts, steps, "obp", root), (volts, Bz - 1e-4, parts, steps, "obm", root)]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(_oracle_loss_worker, jobs)
    for q, k in enumerate((2, 5)):
        (lp, np_), (lm, nm) = res[2 * q], res[2 * q + 1]
        assert np_ == nm, (k, np_, nm)
        fd = (lp - lm) / 2e-3
        assert abs(grad[k] - fd) <= 1e-3 * max(abs(fd), 0.05 * scale), (k, grad[k], fd)
    (lp, np_), (lm, nm) = res[4], res[5]
    assert np_ == nm
    fd = (lp - lm) / 2e-4
    assert abs(grad[10] - fd) <= 1e-3 * abs(fd) + 1e-6, (grad[10], fd)
