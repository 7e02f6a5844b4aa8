"""Batched instances (mag_batch_*) against the same instances run one by one.

The batched kernels run the per-particle, per-node and per-candidate code of
the single-instance kernels, and no launch parameter changes a result, so a
batched run and the separate runs of its instances agree bit for bit: the
particles (matched by id), the collision counters and the potential.  The
separate runs use the multigrid solve as the batch does (a single small
instance would otherwise solve with the precomputed inverse, equal only to
the solver tolerance).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def m(built):
    import mag2d_gb300

    return mag2d_gb300


def _state(pic):
    sp = pic.speclist[0]
    g = sp.particles()
    order = np.argsort(g["id"])
    return {k: v[order] for k, v in g.items()}, sp.diag(), pic.field.u


def _compare(a, b, tag):
    ga, da, ua = a
    gb, db, ub = b
    for k in ("id", "x", "z", "vx", "vy", "vz"):
        assert np.array_equal(ga[k], gb[k]), (tag, k)
    for k in ("n_live", "collisions", "null_collisions", "removed", "particle_steps", "niter"):
        assert da[k] == db[k], (tag, k, da[k], db[k])
    assert np.array_equal(ua, ub), tag


@pytest.mark.parametrize("graph", [True, False], ids=["graph", "launches"])
def test_batch_equals_separate_runs(m, tmp_path, graph):
    from cases import batched_penning

    inst = batched_penning(tmp_path, n=5, np_range=(2e3, 2e4), pressure_range=(1e-2, 1e-1))
    steps = 45  # crosses two particle sorts (interval 20)
    b = m.Batch([(c[3], c[4], c[5], c[6]) for c in inst], sort_interval=20)
    b.set_graph(graph)
    b.advance_init()
    b.advance(steps)
    b.sync()
    got = [_state(b[i]) for i in range(len(b))]
    assert sum(g[1]["collisions"] for g in got) > 0
    for i, c in enumerate(inst):
        pic = m.Pic(c[3], c[4], c[5], seed=c[6], sort_interval=20, direct_solve=-1)
        pic.advance_init()
        pic.advance(steps)
        _compare(got[i], _state(pic), i)
        pic.close()
    b.close()


def test_batch_tuner_keeps_results(m, tmp_path):
    """The autotuner times real steps with other launch parameters; the
    instances then hold exactly the state of an untuned run of as many steps."""
    from cases import batched_penning

    inst = batched_penning(tmp_path, n=3, np_range=(1e3, 5e3))
    b = m.Batch([(c[3], c[4], c[5], c[6]) for c in inst])
    b.advance_init()
    t = b.tune(2)
    assert t["push_vec"] in (1, 2, 4) and t["solve_threads"] in (256, 512, 1024)
    assert t["sort_interval"] in (10, 20, 50) and t["ms_per_step"] > 0
    b.advance(7)
    b.sync()
    steps = b[0].speclist[0].diag()["niter"]
    got = [_state(b[i]) for i in range(len(b))]
    for i, c in enumerate(inst):
        pic = m.Pic(c[3], c[4], c[5], seed=c[6], direct_solve=-1)
        pic.advance_init()
        pic.advance(int(steps))
        _compare(got[i], _state(pic), i)
        pic.close()
    b.close()
