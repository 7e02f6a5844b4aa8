"""Python mirror of the reference's Pic / Fields / Species interface
(src/pic.cpp:115-538, src/fields.hpp:187-222, src/particles.hpp:95-318) over
the C ABI of libmag2d_gpu.so.

    pic = Pic("config.txt", "species_conf.txt", initscript="initscript.txt", seed=1)
    pic.advance_init()
    for i in range(niter):
        pic.advance()
    u = pic.field.u                      # Field2D data as a numpy (x, z) array
    e = pic.speclist["ELECTRON"]         # Species view
    p = e.particles()                    # dict of SoA numpy arrays in SI units

The compute happens on the GPU; this module only moves data and arguments.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import (MAG_MASK, MAG_RHO, MAG_SPECIES_RHO, MAG_U, MAG_URF, MAG_VOLTAGE, MagDiag, MagOpts,
                   MagSolveInfo, MagSpeciesInfo, check, lib)

_D = ctypes.POINTER(ctypes.c_double)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


class Fields:
    """The Fields members u, uRF, rho and the t_grid mask/voltage, as numpy copies."""

    def __init__(self, pic: "Pic"):
        self._pic = pic

    def _get(self, which: int) -> np.ndarray:
        nx, nz = self._pic.shape if which not in (MAG_MASK, MAG_VOLTAGE) else self._pic.mask_shape
        out = np.zeros((nx, nz))
        check(lib().mag_get_field(self._pic.h, which, _dp(out)))
        return out

    @property
    def u(self) -> np.ndarray:
        return self._get(MAG_U)

    @property
    def uRF(self) -> np.ndarray:
        return self._get(MAG_URF)

    @property
    def rho(self) -> np.ndarray:
        return self._get(MAG_RHO)

    @property
    def mask(self) -> np.ndarray:
        return self._get(MAG_MASK).astype(np.int8)

    @property
    def voltage(self) -> np.ndarray:
        return self._get(MAG_VOLTAGE)

    @property
    def faces(self) -> tuple[np.ndarray, np.ndarray]:
        """The FP32 face field the particle kernel reads: Ex ((nx+1, nz)) and Ez ((nx, nz+1))."""
        nx, nz = self._pic.shape
        ex = np.zeros((nx + 1, nz), dtype=np.float32)
        ez = np.zeros((nx, nz + 1), dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        check(lib().mag_get_face_field(self._pic.h, 0, ex.ctypes.data_as(fp)))
        check(lib().mag_get_face_field(self._pic.h, 1, ez.ctypes.data_as(fp)))
        return ex, ez

    def set_rho(self, rho: np.ndarray) -> None:
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        check(lib().mag_set_field(self._pic.h, MAG_RHO, _dp(rho)))

    def set_u(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, dtype=np.float64)
        check(lib().mag_set_field(self._pic.h, MAG_U, _dp(u)))

    def boundary_solve(self, rho: np.ndarray | None = None) -> dict:
        """Fields::boundary_solve (src/fields.cpp:278-312) of the given or current rho."""
        if rho is not None:
            self.set_rho(rho)
        info = MagSolveInfo()
        check(lib().mag_field_solve(self._pic.h, ctypes.byref(info)))
        return {"iterations": info.iterations, "residual": info.residual, "status": info.status,
                "levels": info.levels}


class Species:
    """View of one species (BaseSpecies / Species<D>)."""

    def __init__(self, pic: "Pic", index: int):
        self._pic = pic
        self.index = index

    def info(self) -> dict:
        s = MagSpeciesInfo()
        check(lib().mag_species(self._pic.h, self.index, ctypes.byref(s)))
        return {k: (getattr(s, k).decode() if k == "name" else getattr(s, k)) for k, _ in s._fields_}

    @property
    def name(self) -> str:
        return self.info()["name"]

    def n_particles(self) -> int:
        return int(self.info()["n_live"])

    def particles(self) -> dict:
        """Live particles as SoA numpy arrays: x, z [m], vx, vy, vz [m/s], id."""
        cap = max(int(self.info()["capacity"]), 1)
        arrs = {k: np.zeros(cap) for k in ("x", "z", "vx", "vy", "vz")}
        ids = np.zeros(cap, dtype=np.uint32)
        n = ctypes.c_int64()
        check(lib().mag_get_particles(self._pic.h, self.index, cap, *[_dp(arrs[k]) for k in ("x", "z", "vx", "vy", "vz")],
                                      ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(n)))
        out = {k: v[: n.value].copy() for k, v in arrs.items()}
        out["id"] = ids[: n.value].copy()
        return out

    def set_particles(self, x, z, vx, vy, vz) -> None:
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (x, z, vx, vy, vz)]
        check(lib().mag_set_particles(self._pic.h, self.index, len(a[0]), *[_dp(v) for v in a]))

    def diag(self) -> dict:
        d = MagDiag()
        check(lib().mag_diag(self._pic.h, self.index, ctypes.byref(d)))
        return {k: getattr(d, k) for k, _ in d._fields_}

    def energy_dist(self) -> dict:
        """Sampled energy histogram (Histogram::print values) and its statistics."""
        c, v, st = np.zeros(200), np.zeros(200), np.zeros(4)
        n = check(lib().mag_energy_dist(self._pic.h, self.index, 200, _dp(c), _dp(v), _dp(st)))
        return {"centers": c[:n], "values": v[:n], "n_val": st[0], "mean": st[1] / st[0] if st[0] else 0.0,
                "n_val_tot": st[2], "mean_tot": st[3] / st[2] if st[2] else 0.0}

    @property
    def rho_average(self) -> np.ndarray:
        out = np.zeros(self._pic.shape)
        check(lib().mag_get_average(self._pic.h, MAG_SPECIES_RHO + self.index, _dp(out)))
        return out

    def save(self, path) -> None:
        """BaseSpecies::save (src/particles.cpp:32-57)."""
        check(lib().mag_species_save(self._pic.h, self.index, str(path).encode()))

    def load(self, path) -> None:
        """BaseSpecies::load (src/particles.cpp:59-93)."""
        check(lib().mag_species_load(self._pic.h, self.index, str(path).encode()))

    def n_live(self) -> int:
        """BaseSpecies::n_particles (src/particles.hpp:248)."""
        n = ctypes.c_int64()
        check(lib().mag_n_live(self._pic.h, self.index, ctypes.byref(n)))
        return n.value

    def particles_aos(self) -> np.ndarray:
        """Live particles as t_particle records (x, y, z, vx, vy, vz, time_to_death, empty)."""
        cap = max(int(self.info()["capacity"]), 1)
        rec = np.zeros((cap, 8), dtype=np.float64)
        n = ctypes.c_int64()
        check(lib().mag_get_particles_aos(self._pic.h, self.index, cap, rec.ctypes.data_as(ctypes.c_void_p),
                                          ctypes.byref(n)))
        return rec[: n.value].copy()

    def source_save(self, path) -> None:
        """BaseSpecies::source5_save (src/particles.cpp:109-120)."""
        check(lib().mag_source_save(self._pic.h, self.index, str(path).encode()))

    def source_load(self, path) -> None:
        """BaseSpecies::source5_load (src/particles.cpp:122-140)."""
        check(lib().mag_source_load(self._pic.h, self.index, str(path).encode()))

    def source_info(self) -> dict:
        """Source box particles, copies appended to the species so far, copies dropped."""
        v = [ctypes.c_int64() for _ in range(3)]
        check(lib().mag_source_info(self._pic.h, self.index, *[ctypes.byref(x) for x in v]))
        return {"n_box": v[0].value, "injected": v[1].value, "dropped": v[2].value}

    def rho_fixed(self) -> np.ndarray:
        nx, nz = self._pic.shape
        out = np.zeros((nx, nz), dtype=np.int64)
        check(lib().mag_get_rho_fixed(self._pic.h, self.index, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    @property
    def rho(self) -> np.ndarray:
        return self._pic.field._get(MAG_SPECIES_RHO + self.index)


class Speclist:
    def __init__(self, pic: "Pic"):
        self._pic = pic
        self._sp = [Species(pic, i) for i in range(check(lib().mag_n_species(pic.h)))]

    def __len__(self) -> int:
        return len(self._sp)

    def __iter__(self):
        return iter(self._sp)

    def __getitem__(self, key):
        if isinstance(key, str):
            for s in self._sp:
                if s.name == key:
                    return s
            raise KeyError(key)
        return self._sp[key]


class Pic:
    """Pic<D> of the reference, on the GPU."""

    def __init__(self, config, species_conf, initscript=None, *, seed: int = 1, device: int = 0,
                 poisson_tol: float = 0.0, poisson_max_iter: int = 0, capacity_hint: int = 0,
                 sort_interval: int = 0, push_vec: int = 0, direct_solve: int = 0, max_fused_steps: int = 0,
                 multigrid_fp64: int = 0):
        opts = MagOpts(device=device, seed=seed, sort_interval=sort_interval, poisson_tol=poisson_tol,
                       poisson_max_iter=poisson_max_iter, capacity_hint=capacity_hint, push_vec=push_vec,
                       direct_solve=direct_solve, max_fused_steps=max_fused_steps, multigrid_fp64=multigrid_fp64)
        h = ctypes.c_void_p()
        ini = str(initscript).encode() if initscript else None
        check(lib().mag_create(str(config).encode(), str(species_conf).encode(), ini, ctypes.byref(opts),
                               ctypes.byref(h)))
        self._attach(h, config)

    @classmethod
    def _borrowed(cls, h, config) -> "Pic":
        """View of an instance that a Batch owns (not closed by this object)."""
        obj = cls.__new__(cls)
        obj._attach(h, config)
        obj._owned = False
        return obj

    def _attach(self, h, config) -> None:
        self.h = h
        self._owned = True
        nx, nz = ctypes.c_int(), ctypes.c_int()
        dx, dz, x0, z0 = (ctypes.c_double() for _ in range(4))
        check(lib().mag_grid(self.h, ctypes.byref(nx), ctypes.byref(nz), ctypes.byref(dx), ctypes.byref(dz),
                             ctypes.byref(x0), ctypes.byref(z0)))
        self.shape = (nx.value, nz.value)
        self.dx, self.dz, self.x_min, self.z_min = dx.value, dz.value, x0.value, z0.value
        self.mask_shape = (int(config_param(config, "x_sampl")), int(config_param(config, "z_sampl")))
        self.field = Fields(self)
        self.speclist = Speclist(self)

    def close(self) -> None:
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                lib().mag_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run_initscript(self, path) -> None:
        check(lib().mag_run_initscript(self.h, str(path).encode()))

    def advance_init(self) -> None:
        check(lib().mag_advance_init(self.h))

    def advance(self, n: int = 1) -> None:
        check(lib().mag_advance(self.h, n))

    def set_electrode_voltages(self, v: np.ndarray) -> None:
        """t_grid::voltage of the fixed nodes (x_sampl, z_sampl); the fields follow."""
        a = np.ascontiguousarray(v, dtype=np.float64)
        check(lib().mag_set_electrode_voltages(self.h, _dp(a), a.size))

    def source_refresh(self, factor: int) -> None:
        """Species<CARTESIAN>::source5_refresh(factor) of every species with particles."""
        check(lib().mag_source_refresh(self.h, factor))

    def advance_timed(self, n: int = 1):
        """advance(n) with CUDA event timing: (sort_ms, solve_ms, particle_ms, collide_ms)."""
        ms = np.zeros(4)
        check(lib().mag_advance_timed(self.h, n, _dp(ms)))
        return tuple(ms)

    def dist_reset(self) -> None:
        check(lib().mag_dist_reset(self.h))

    def dist_sample(self) -> None:
        check(lib().mag_dist_sample(self.h))

    @property
    def u_average(self) -> np.ndarray:
        out = np.zeros(self.shape)
        check(lib().mag_get_average(self.h, MAG_U, _dp(out)))
        return out

    def print_distribution(self, directory) -> None:
        check(lib().mag_print_distribution(self.h, str(directory).encode()))

    def print_field(self, path) -> None:
        check(lib().mag_print_field(self.h, str(path).encode()))

    def print_trace(self, directory) -> None:
        """Pic::print_trace: one "x z vx vz vy" line per tracked particle
        (add_tracked_particle) appended to <dir>/<species>_traj_<slot>.dat."""
        check(lib().mag_print_trace(self.h, str(directory).encode()))

    def solve_status(self) -> dict:
        """Status of the most recent Poisson solve (iterations, residual, status, levels)."""
        info = MagSolveInfo()
        check(lib().mag_solve_status(self.h, ctypes.byref(info)))
        return {"iterations": info.iterations, "residual": info.residual, "status": info.status,
                "levels": info.levels}

    def solve_phase_times(self) -> dict:
        """Phase times [ms] of the most recent multigrid solve (mag_solve_phase_times);
        the first call switches the timing on and returns zeros."""
        out = np.zeros(29)
        n = check(lib().mag_solve_phase_times(self.h, _dp(out), len(out)))
        out = out[:n]
        return {"start": out[0], "residual": out[1], "down": list(out[2:14]), "coarse": out[14],
                "up": list(out[15:27]), "faces": out[27], "total": out[28]}

    def adjoint(self, nsteps: int, voltage_keys=(), *, checkpoint: int = 100, grad_b: bool = True,
                w_energy: float = 1.0, w_lost: float = 1.0):
        """mag_adjoint_run: runs advance_init and nsteps steps, returns (info, gradient).

        gradient = d loss / d(voltage_keys...) followed by d loss / d(Br, Bt, Bz) when grad_b;
        loss = w_energy * mean axial kinetic energy [eV] + w_lost * lost fraction."""
        from ._lib import MagAdjCfg, MagAdjOut

        keys = [str(k).encode() for k in voltage_keys]
        arr = (ctypes.c_char_p * max(1, len(keys)))(*keys)
        cfg = MagAdjCfg(nsteps=nsteps, checkpoint=checkpoint, n_voltage_keys=len(keys), voltage_keys=arr,
                        grad_b=1 if grad_b else 0, w_energy=w_energy, w_lost=w_lost)
        grad = np.zeros(len(keys) + (3 if grad_b else 0))
        out = MagAdjOut()
        check(lib().mag_adjoint_run(self.h, ctypes.byref(cfg), _dp(grad), ctypes.byref(out)))
        info = {"loss": out.loss, "mean_energy_eV": out.mean_energy_eV, "lost_fraction": out.lost_fraction,
                "n0": out.n0, "n_live": out.n_live}
        return info, grad

    def sync(self) -> None:
        check(lib().mag_sync(self.h))

    def deposit(self) -> None:
        check(lib().mag_deposit(self.h))

    @property
    def stream(self) -> int:
        return lib().mag_stream(self.h) or 0

    @property
    def kernel_launches(self) -> int:
        return int(lib().mag_kernel_launches(self.h))


def read_particle_file(path) -> dict:
    """The particles of a BaseSpecies::save file (host only, no GPU)."""
    n, total = ctypes.c_int64(), ctypes.c_int64()
    check(lib().mag_particle_file_read(str(path).encode(), 0, *([None] * 7), ctypes.byref(n), ctypes.byref(total)))
    out = {k: np.zeros(n.value) for k in ("x", "y", "z", "vx", "vy", "vz", "time_to_death")}
    check(lib().mag_particle_file_read(str(path).encode(), n.value, *[_dp(out[k]) for k in out], ctypes.byref(n),
                                       ctypes.byref(total)))
    out["total"] = total.value
    return out


def write_particle_file(path, x, z, vx, vy, vz, *, y=None, time_to_death=None, total: int = 0) -> None:
    """Write particles in the BaseSpecies::save format (host only, no GPU)."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, z, vx, vy, vz)]
    n = len(arrs[0])
    yy = None if y is None else np.ascontiguousarray(y, dtype=np.float64)
    tt = None if time_to_death is None else np.ascontiguousarray(time_to_death, dtype=np.float64)
    check(lib().mag_particle_file_write(str(path).encode(), int(total), n, _dp(arrs[0]),
                                        None if yy is None else _dp(yy), _dp(arrs[1]), _dp(arrs[2]), _dp(arrs[3]),
                                        _dp(arrs[4]), None if tt is None else _dp(tt)))


def config_param(config, key: str) -> float:
    """Param value of a config file (host-only, no GPU)."""
    v = ctypes.c_double()
    check(lib().mag_config_param(str(config).encode(), key.encode(), ctypes.byref(v)))
    return v.value


def config_geometry(config):
    """(mask, voltage) of the config's geometry (host-only, no GPU)."""
    nx, nz = ctypes.c_int(), ctypes.c_int()
    nx_ = int(config_param(config, "x_sampl"))
    nz_ = int(config_param(config, "z_sampl"))
    mask = np.zeros((nx_, nz_), dtype=np.int8)
    volt = np.zeros((nx_, nz_))
    check(lib().mag_config_geometry(str(config).encode(), nx_ * nz_,
                                    mask.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), _dp(volt),
                                    ctypes.byref(nx), ctypes.byref(nz)))
    return mask, volt


def config_species(config, species_conf, index: int):
    """(info dict, rates array) of species 'index' (host-only, no GPU)."""
    info = MagSpeciesInfo()
    rates = np.zeros(64)
    n = check(lib().mag_config_species(str(config).encode(), str(species_conf).encode(), index,
                                       ctypes.byref(info), _dp(rates)))
    d = {k: (getattr(info, k).decode() if k == "name" else getattr(info, k)) for k, _ in info._fields_}
    return d, rates[:n]


class Batch:
    """Many independent Pic instances advanced together (mag_batch_* of the C ABI).

    instances: sequence of (config, species_conf, initscript or None, seed).
    """

    def __init__(self, instances, *, device: int = 0, poisson_tol: float = 0.0, poisson_max_iter: int = 0,
                 capacity_hint: int = 0, sort_interval: int = 0, push_vec: int = 0):
        from ._lib import MagInstanceDesc

        opts = MagOpts(device=device, seed=0, sort_interval=sort_interval, poisson_tol=poisson_tol,
                       poisson_max_iter=poisson_max_iter, capacity_hint=capacity_hint, push_vec=push_vec)
        inst = list(instances)
        self._keep = []
        arr = (MagInstanceDesc * len(inst))()
        for i, (cfg, spc, ini, seed) in enumerate(inst):
            c, sc, ic = str(cfg).encode(), str(spc).encode(), (str(ini).encode() if ini else None)
            self._keep += [c, sc, ic]
            arr[i].config_path, arr[i].species_conf_path, arr[i].initscript_path, arr[i].seed = c, sc, ic, int(seed)
        h = ctypes.c_void_p()
        check(lib().mag_batch_create(len(inst), arr, ctypes.byref(opts), ctypes.byref(h)))
        self.h = h
        self.instances = []
        for i, (cfg, _, _, _) in enumerate(inst):
            v = ctypes.c_void_p()
            check(lib().mag_batch_instance(self.h, i, ctypes.byref(v)))
            self.instances.append(Pic._borrowed(v, cfg))

    def __len__(self) -> int:
        return len(self.instances)

    def __getitem__(self, i) -> Pic:
        return self.instances[i]

    def advance_init(self) -> None:
        check(lib().mag_batch_advance_init(self.h))

    def advance(self, n: int = 1) -> None:
        check(lib().mag_batch_advance(self.h, n))

    def tune(self, steps_per_trial: int = 3) -> dict:
        from ._lib import MagBatchTuning

        t = MagBatchTuning()
        check(lib().mag_batch_tune(self.h, steps_per_trial, ctypes.byref(t)))
        return {"push_vec": t.push_vec, "solve_threads": t.solve_threads, "sort_interval": t.sort_interval,
                "ms_per_step": t.ms_per_step}

    def set_graph(self, enabled: bool) -> None:
        check(lib().mag_batch_set_graph(self.h, 1 if enabled else 0))

    def sync(self) -> None:
        check(lib().mag_batch_sync(self.h))

    @property
    def stream(self) -> int:
        return lib().mag_batch_stream(self.h) or 0

    @property
    def kernel_launches(self) -> int:
        return int(lib().mag_batch_kernel_launches(self.h))

    def close(self) -> None:
        if getattr(self, "h", None):
            for p in self.instances:
                p.h = None
            lib().mag_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pic3D:
    """The 3D Cartesian run (coord = CARTESIAN3D): ElMag3D + Species<CARTESIAN3D>
    of the reference (src/fields3d.cpp, src/species3d.cpp, src/Field3D.hpp) on
    the GPU.  Arrays of nodes are (nx, ny, nz), z fastest."""

    def __init__(self, config, species_conf, *, seed: int = 1, device: int = 0, poisson_tol: float = 0.0,
                 poisson_max_iter: int = 0, capacity_hint: int = 0):
        opts = MagOpts(device=device, seed=seed, poisson_tol=poisson_tol, poisson_max_iter=poisson_max_iter,
                       capacity_hint=capacity_hint)
        h = ctypes.c_void_p()
        check(lib().mag3d_create(str(config).encode(), str(species_conf).encode(), ctypes.byref(opts),
                                 ctypes.byref(h)))
        self.h = h
        dims = (ctypes.c_int * 3)()
        sp = np.zeros(3)
        self.nspecies = check(lib().mag3d_grid(self.h, dims, _dp(sp)))
        self.shape = (dims[0], dims[1], dims[2])
        self.spacing = tuple(sp)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().mag3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, species: int, x, y, z, vx, vy, vz) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, vx, vy, vz)]
        check(lib().mag3d_set_particles(self.h, species, len(arrs[0]), *[_dp(a) for a in arrs]))

    def particles(self, species: int) -> dict:
        cap = max(int(self.diag(species)["n_live"]), 1)
        n = ctypes.c_int64()
        arrs = {k: np.zeros(cap) for k in ("x", "y", "z", "vx", "vy", "vz")}
        ids = np.zeros(cap, dtype=np.uint32)
        check(lib().mag3d_get_particles(self.h, species, cap, *[_dp(arrs[k]) for k in ("x", "y", "z", "vx", "vy", "vz")],
                                        ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(n)))
        out = {k: v[: n.value].copy() for k, v in arrs.items()}
        out["id"] = ids[: n.value].copy()
        return out

    def advance_init(self) -> None:
        check(lib().mag3d_advance_init(self.h))

    def advance(self, n: int = 1) -> None:
        check(lib().mag3d_advance(self.h, n))

    def solve(self, rho: np.ndarray | None = None) -> dict:
        """ElMag3D::solve of a charge density [C/m^3] (nx, ny, nz), or of the deposits."""
        info = MagSolveInfo()
        r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
        rc = lib().mag3d_solve(self.h, _dp(r) if r is not None else None, ctypes.byref(info))
        if rc not in (0, -4):
            check(rc)
        return {"iterations": info.iterations, "residual": info.residual, "status": info.status}

    def field(self, which: int = MAG_U) -> np.ndarray:
        out = np.zeros(self.shape)
        check(lib().mag3d_get_field(self.h, which, _dp(out)))
        return out

    @property
    def u(self) -> np.ndarray:
        return self.field(MAG_U)

    def rho_fixed(self, species: int) -> np.ndarray:
        out = np.zeros(self.shape, dtype=np.int64)
        check(lib().mag3d_get_rho_fixed(self.h, species, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    def diag(self, species: int) -> dict:
        d = MagDiag()
        check(lib().mag3d_diag(self.h, species, ctypes.byref(d)))
        return {k: getattr(d, k) for k, _ in d._fields_}

    @property
    def kernel_launches(self) -> int:
        return int(lib().mag3d_kernel_launches(self.h))
