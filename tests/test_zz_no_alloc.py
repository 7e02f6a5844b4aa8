"""The allocation-free Poisson solve (mag_poisson_solve_noalloc) against the
regular one (mag_field_solve through a simulation handle).

Callers of the no-allocation entry point cannot call cudaMalloc themselves
(fixed device-memory budgets, allocators they do not own), so the library
must run the whole multigrid solve in its static scratch array.  These tests
call it through the C ABI several times in a row — each call reuses the
scratch array the previous one left behind — on a cylindrical and a Cartesian
grid, and check each result against the regular solve of the same charge
density, within the 1e-9 relative tolerance of the other Poisson parity
tests.  The file sorts last so that a run stopping at
the first failure has already run every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


GEOMETRIES = {
    "cylindrical": dict(coord="CYLINDRICAL", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3, r_sampl=65,
                        z_sampl=129),
    "cartesian": dict(coord="CARTESIAN", geometry="PROBE", x_max=2e-2, z_max=2e-2, x_sampl=65, z_sampl=65,
                      probe_radius=1e-3),
}


@pytest.mark.parametrize("geom", list(GEOMETRIES), ids=list(GEOMETRIES))
def test_noalloc_solve_matches_field_solve(built, tmp_path, geom):
    """Three calls in a row, each checked against the regular solve of the
    same charge density: two that wait and report (info given), then one that
    only queues the work (info NULL) and is read after a device
    synchronisation.  The free device memory is the same before and after the
    second call: the entry point allocates nothing (the first call may still
    load the solve kernel's module, so it is not the one measured)."""
    torch = pytest.importorskip("torch")
    import mag2d_gb300 as m
    from mag2d_cases import QE, write_config, write_species_conf
    from mag2d_gb300._lib import MagSolveInfo, lib

    cfg = dict(selfconsistent=1, rf=0, do_plot=0, macroparticle_factor=100.0, **GEOMETRIES[geom])
    coord = 1 if cfg["coord"] == "CYLINDRICAL" else 0
    sp = [dict(name="E", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, temperature=1e4, density=1e13)]
    cpath = write_config(cfg, tmp_path / "c.txt")
    spath = write_species_conf(sp, [], tmp_path / "s.txt")
    pic = m.Pic(cpath, spath, seed=1, direct_solve=-1)
    mask, volt = m.config_geometry(cpath)
    nx, nz = pic.shape
    dV = m.config_param(cpath, "dV")
    L = lib()
    L.mag_poisson_solve_noalloc.argtypes = [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
        ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(MagSolveInfo)]
    mask = np.ascontiguousarray(mask, dtype=np.int8)
    volt = np.ascontiguousarray(volt, dtype=np.float64)
    rng = np.random.default_rng(7)
    u_dev = torch.zeros((nx, nz), dtype=torch.float64, device="cuda")
    for trial in range(3):
        rho = -QE * 10 * rng.random((nx, nz)) * (1 + trial)
        pic.field.boundary_solve(rho)
        u_ref = pic.field.u
        rho_dev = torch.tensor(rho, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        info = MagSolveInfo() if trial < 2 else None
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.mag_poisson_solve_noalloc(coord, nx, nz, pic.dx, pic.dz, 100.0, dV, mask.ctypes.data,
                                        volt.ctypes.data, rho_dev.data_ptr(), u_dev.data_ptr(), 1e-12, 200, None,
                                        ctypes.byref(info) if info is not None else None)
        assert rc == 0, L.mag_last_error()
        torch.cuda.synchronize()
        if trial == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        if info is not None:
            assert info.status == 0 and info.levels > 1, (info.status, info.levels)
        u = u_dev.cpu().numpy()
        err = np.abs(u - u_ref).max() / np.abs(u_ref).max()
        assert err <= 1e-9, (geom, trial, err)
    pic.close()


def test_noalloc_rejects_grids_above_the_limit(built):
    pytest.importorskip("torch")
    from mag2d_gb300._lib import lib

    L = lib()
    n = 300
    mask = np.full((n, n), 2, dtype=np.int8)
    volt = np.zeros((n, n))
    rc = L.mag_poisson_solve_noalloc(0, n, n, ctypes.c_double(1e-4), ctypes.c_double(1e-4), ctypes.c_double(1.0),
                                    ctypes.c_double(1.0), mask.ctypes.data, volt.ctypes.data, ctypes.c_void_p(16),
                                    ctypes.c_void_p(16), ctypes.c_double(1e-12), 200, None, None)
    assert rc == -1
    assert b"257 x 257" in L.mag_last_error()
