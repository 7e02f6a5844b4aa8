"""Test-side helpers: case definitions, input-file writers and ctypes bindings
of the two CPU checkers (the oracle port and, where it was built here, the
reference compiled from its own sources).

Only tests, the golden-fixture script, ``__graft_entry__.smoke`` and the
``cpu_baseline`` leg of ``bench.py`` use this module.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PORT_SO = ROOT / "oracle" / "build" / "libmag2d_oracle.so"
# the same port built with the reference's -Ofast, for CPU-baseline timing only
PORT_TIMING_SO = ROOT / "oracle" / "build" / "libmag2d_oracle_timing.so"
REF_SO = ROOT / "oracle" / "_ref" / "libmag2d_ref.so"

# Physical constants of the reference (src/param.cpp:8-10)
EPS0 = 8.854187817e-12
KB = 1.380662e-23
QE = 1.602189e-19
AMU = 1.66054e-27

# Defaults of Param (src/param.cpp:14-143) for the keys the tests set
PARAM_DEFAULTS = {
    "coord": "CYLINDRICAL", "boundary": "FREE", "geometry": "EMPTY",
    "x_max": 1e-2, "y_max": 1e-2, "z_max": 1e-2, "x_sampl": 100, "z_sampl": 100,
    "n_particles_total": 1e5, "density_total": 1e11, "macroparticle_factor": 1e4,
    "extern_field": 100.0, "selfconsistent": 1, "rf": 1, "rf_amplitude": 10.0,
    "rf_U0": 0.0, "rf_freq": 20e6, "electric_field_from_file": 0,
    "magnetic_field_const": 1, "Br": 0.0, "Bz": 0.0, "Bt": 0.0, "do_plot": 0,
    "mover": "ADVANCE_BORIS", "u_probe": -10.0, "probe_radius": 1e-4, "u_smooth": 0,
}

COLL_TYPES = {"ELASTIC": 0, "LANGEVIN": 1, "CX": 2, "COULOMB": 3, "SUPERELASTIC": 4}


def full_config(cfg: dict) -> dict:
    """Config with the reference defaults filled in (x_max/x_sampl aliases resolved)."""
    out = dict(PARAM_DEFAULTS)
    out.update(cfg)
    if "r_max" in cfg and "x_max" not in cfg:
        out["x_max"] = cfg["r_max"]
    if "r_sampl" in cfg and "x_sampl" not in cfg:
        out["x_sampl"] = cfg["r_sampl"]
    if "rf_omega" not in out:
        out["rf_omega"] = 2 * np.pi * float(out["rf_freq"])
    return out


def poisson_system(cfg: dict, mask: np.ndarray, volt: np.ndarray, rho: np.ndarray):
    """The reference's linear system of Fields::boundary_solve (src/fields.cpp:136-312):
    the 5-point row stencil of every free node (cylindrical axis row at i = 0),
    identity rows at fixed nodes, the right-hand side scaled as the reference
    scales rho.  Vectorised; returns (A as scipy CSR, b)."""
    import scipy.sparse as sp

    c = full_config(cfg)
    nx, nz = mask.shape
    dx, dz = float(c["x_max"]) / (nx - 1), float(c["z_max"]) / (nz - 1)
    cyl = c["coord"] == "CYLINDRICAL"
    N = nx * nz
    k = np.arange(N).reshape(nx, nz)
    i = np.broadcast_to(np.arange(nx)[:, None], (nx, nz))
    fixed = (mask == 0) | (mask == 1)
    free = ~fixed
    b = np.zeros(N)
    rows, cols, vals = [k[fixed]], [k[fixed]], [np.ones(int(fixed.sum()))]
    b[k[fixed]] = np.where(mask[fixed] == 0, volt[fixed], 0.0)
    mpf = float(c["macroparticle_factor"])
    if cyl:
        ax = free & (i == 0)
        ka = k[ax]
        k2, k3 = 1 / dz ** 2, 1 / (dx * dx * 0.25)
        for off, v in ((-1, k2), (0, -2 * k2 - k3), (1, k2), (nz, k3)):
            rows.append(ka), cols.append(ka + off), vals.append(np.full(len(ka), v))
        b[ka] = rho[ax] * (-1.0 / EPS0 / (np.pi * dx * dx * 0.25 * dz) * mpf)
        inn = free & (i > 0)
        ki, ii = k[inn], i[inn].astype(float)
        k1, k3 = (ii - 0.5) / (dx * dx * ii), (ii + 0.5) / (dx * dx * ii)
        for off, v in ((-nz, k1), (-1, np.full(len(ki), k2)), (0, -2 * k2 - k1 - k3), (1, np.full(len(ki), k2)),
                       (nz, k3)):
            rows.append(ki), cols.append(ki + off), vals.append(v)
        b[ki] = rho[inn] * (-1.0 / EPS0 / (np.pi * dx * dx * 2.0 * ii * dz) * mpf)
    else:
        kf = k[free]
        V = float(c["n_particles_total"]) / float(c["density_total"])
        dV = V / ((nx - 1) * (nz - 1))
        for off, v in ((-nz, 1.0), (-1, 1.0), (0, -4.0), (1, 1.0), (nz, 1.0)):
            rows.append(kf), cols.append(kf + off), vals.append(np.full(len(kf), v))
        b[kf] = rho[free] * (-dx * dx / EPS0 / dV)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    return A, b


def write_config(cfg: dict, path) -> Path:
    """Write a GetPot-style config.txt (key = value lines)."""
    path = Path(path)
    lines = ["# generated test configuration"]
    for k, v in cfg.items():
        if isinstance(v, (float, np.floating)):
            v = repr(float(v))
        elif isinstance(v, (np.integer,)):
            v = int(v)
        lines.append(f"{k} = {v}")
    path.write_text("\n".join(lines) + "\n")
    return path


def write_species_conf(species: list, interactions: list, path) -> Path:
    """Write a species_conf file in the block format of src/parser.cpp:25-147."""
    path = Path(path)
    out = []
    keys = [("name", "NAME"), ("dt", "DT"), ("type", "TYPE"), ("mass", "MASS"),
            ("charge", "CHARGE"), ("density", "DENSITY"), ("temperature", "TEMPERATURE"),
            ("emax", "EMAX")]
    for s in species:
        out.append("SPECIES")
        for k, tag in keys:
            if k in s:
                v = s[k]
                out.append(f"    {tag} {float(v)!r}" if isinstance(v, (float, np.floating)) else f"    {tag} {v}")
        out.append("")
    for it in interactions:
        out.append("INTERACTION")
        out.append(f"    NAME {it['name']}")
        out.append(f"    TYPE {it['type']}")
        out.append(f"    PRIMARY {it['primary']}")
        out.append(f"    SECONDARY {it['secondary']}")
        for k, tag in (("DE", "DE"), ("rate", "RATE"), ("cutoff", "CUTOFF")):
            if k in it:
                out.append(f"    {tag} {float(it[k])!r}")
        if it.get("table"):
            out.append("    CROSS_SECTION")
            for e, sg in it["table"]:
                out.append(f"        {float(e)!r} {float(sg)!r}")
            out.append("    END_CROSS_SECTION")
        out.append("")
    path.write_text("\n".join(out) + "\n")
    return path


def write_field_file(path, x, z, values) -> Path:
    """Write a Field2D::load table (src/Field2D.cpp:46-130): 'x z value' lines, x outer."""
    path = Path(path)
    with open(path, "w") as f:
        for i, xv in enumerate(x):
            for j, zv in enumerate(z):
                f.write(f"{float(xv)!r} {float(zv)!r} {float(values[i, j])!r}\n")
    return path


# ----------------------------------------------------------------------------
# ctypes: oracle port
# ----------------------------------------------------------------------------
class OrcConfig(ctypes.Structure):
    _fields_ = [
        ("coord", ctypes.c_int), ("x_sampl", ctypes.c_int), ("z_sampl", ctypes.c_int),
        ("x_max", ctypes.c_double), ("z_max", ctypes.c_double), ("y_max", ctypes.c_double),
        ("n_particles_total", ctypes.c_double), ("density_total", ctypes.c_double),
        ("macroparticle_factor", ctypes.c_double), ("extern_field", ctypes.c_double),
        ("geometry_empty", ctypes.c_int), ("selfconsistent", ctypes.c_int), ("rf", ctypes.c_int),
        ("electric_field_from_file", ctypes.c_int), ("rf_amplitude", ctypes.c_double),
        ("rf_omega", ctypes.c_double), ("rf_U0", ctypes.c_double), ("boundary", ctypes.c_int),
        ("magnetic_field_const", ctypes.c_int), ("Br", ctypes.c_double), ("Bz", ctypes.c_double),
        ("Bt", ctypes.c_double), ("mover", ctypes.c_int), ("u_smooth", ctypes.c_int),
    ]


_D = ctypes.POINTER(ctypes.c_double)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def load_port(timing: bool = False) -> ctypes.CDLL:
    so = PORT_TIMING_SO if timing else PORT_SO
    if not so.exists():
        raise RuntimeError(f"oracle port not built: {so} (run __graft_entry__.build())")
    L = ctypes.CDLL(str(so))
    L.orc_create.restype = ctypes.c_void_p
    L.orc_create.argtypes = [ctypes.POINTER(OrcConfig), ctypes.c_void_p, ctypes.c_void_p]
    L.orc_last_error.restype = ctypes.c_char_p
    L.orc_time_advance.restype = ctypes.c_double
    L.orc_collisions.restype = ctypes.c_int64
    L.orc_real_collisions.restype = ctypes.c_int64
    L.orc_u_smooth.restype = None
    L.orc_u_smooth.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.orc_deposit_fixed.restype = ctypes.c_int64
    L.orc_deposit_fixed.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    for name in ("orc_destroy", "orc_add_species", "orc_add_interaction", "orc_init", "orc_seed",
                 "orc_run_initscript", "orc_set_particles", "orc_n_slots", "orc_n_live",
                 "orc_get_particles", "orc_advance_init", "orc_advance", "orc_get_field",
                 "orc_field_shape", "orc_solve", "orc_grad", "orc_species_info", "orc_rates",
                 "orc_sigma_v", "orc_rng", "orc_set_loaded_fields", "orc_set_bfield",
                 "orc_time_advance", "orc_collisions"):
        getattr(L, name)
    return L


def orc_config(cfg: dict) -> OrcConfig:
    c = full_config(cfg)
    return OrcConfig(
        coord=1 if c["coord"] == "CYLINDRICAL" else 0,
        x_sampl=int(float(c["x_sampl"])), z_sampl=int(float(c["z_sampl"])),
        x_max=float(c["x_max"]), z_max=float(c["z_max"]), y_max=float(c["y_max"]),
        n_particles_total=float(c["n_particles_total"]), density_total=float(c["density_total"]),
        macroparticle_factor=float(c["macroparticle_factor"]), extern_field=float(c["extern_field"]),
        geometry_empty=1 if c["geometry"] == "EMPTY" else 0,
        selfconsistent=int(float(c["selfconsistent"])), rf=int(float(c["rf"])),
        electric_field_from_file=int(float(c["electric_field_from_file"])),
        rf_amplitude=float(c["rf_amplitude"]), rf_omega=float(c["rf_omega"]), rf_U0=float(c["rf_U0"]),
        boundary=1 if c["boundary"] == "PERIODIC" else 0,
        magnetic_field_const=int(float(c["magnetic_field_const"])),
        Br=float(c["Br"]), Bz=float(c["Bz"]), Bt=float(c["Bt"]),
        mover=1 if str(c.get("mover", "ADVANCE_BORIS")) == "ADVANCE_MULTICOLL" else 0,
        u_smooth=int(float(c.get("u_smooth", 0))),
    )


class Port:
    """The oracle port (oracle/mag2d_oracle.cpp) driven like the reference's Pic."""

    def __init__(self, cfg: dict, species: list, interactions: list, mask: np.ndarray,
                 voltage: np.ndarray, seed: int = 1, loaded_fields=None, timing: bool = False):
        self.L = load_port(timing)
        self.cfg = cfg
        self._c = orc_config(cfg)
        mask = np.ascontiguousarray(mask, dtype=np.int8)
        voltage = np.ascontiguousarray(voltage, dtype=np.float64)
        self.h = ctypes.c_void_p(self.L.orc_create(ctypes.byref(self._c), mask.ctypes.data,
                                                   voltage.ctypes.data))
        self.names = [s["name"] for s in species]
        for s in species:
            self.L.orc_add_species(
                self.h, s["name"].encode(), ctypes.c_double(float(s.get("mass", 0.0))),
                ctypes.c_double(float(s.get("charge", 0.0))), ctypes.c_double(float(s.get("dt", 0.0))),
                ctypes.c_double(float(s.get("density", 0.0))),
                ctypes.c_double(float(s.get("temperature", 0.0))),
                ctypes.c_double(float(s.get("emax", 0.0))))
        for it in interactions:
            tab = np.asarray(it.get("table", []), dtype=np.float64).reshape(-1, 2)
            E = np.ascontiguousarray(tab[:, 0]) if len(tab) else np.zeros(1)
            S = np.ascontiguousarray(tab[:, 1]) if len(tab) else np.zeros(1)
            self.L.orc_add_interaction(
                self.h, self.names.index(it["primary"]), self.names.index(it["secondary"]),
                COLL_TYPES[it["type"]], ctypes.c_double(float(it.get("DE", 0.0))),
                ctypes.c_double(float(it.get("rate", 0.0))), ctypes.c_double(float(it.get("cutoff", 0.0))),
                len(tab), _dp(E), _dp(S))
        if loaded_fields is not None:
            nx, nz, dx, dz, x0, z0, u, urf = loaded_fields
            u = np.ascontiguousarray(u, dtype=np.float64)
            urf = np.ascontiguousarray(urf, dtype=np.float64)
            self._check(self.L.orc_set_loaded_fields(self.h, nx, nz, ctypes.c_double(dx),
                                                     ctypes.c_double(dz), ctypes.c_double(x0),
                                                     ctypes.c_double(z0), _dp(u), _dp(urf)))
        self._check(self.L.orc_init(self.h))
        self.L.orc_seed(self.h, ctypes.c_uint32(seed))

    def _check(self, rc):
        if rc < 0:
            raise RuntimeError(self.L.orc_last_error().decode())
        return rc

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    def set_particles(self, sp: int, x, z, vx, vy, vz):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, z, vx, vy, vz)]
        self._check(self.L.orc_set_particles(self.h, sp, len(arrs[0]), *[_dp(a) for a in arrs]))

    def run_initscript(self, path):
        self._check(self.L.orc_run_initscript(self.h, str(path).encode()))

    def particles(self, sp: int) -> np.ndarray:
        n = self.L.orc_n_slots(self.h, sp)
        out = np.zeros((max(n, 1), 8))
        self.L.orc_get_particles(self.h, sp, _dp(out))
        return out[:n]

    def n_live(self, sp: int) -> int:
        return self.L.orc_n_live(self.h, sp)

    def advance_init(self):
        self._check(self.L.orc_advance_init(self.h))

    def advance(self, n: int = 1):
        self._check(self.L.orc_advance(self.h, n))

    def time_advance(self, n: int) -> float:
        return self.L.orc_time_advance(self.h, n)

    def field(self, which: int) -> np.ndarray:
        nx, nz = ctypes.c_int(), ctypes.c_int()
        self.L.orc_field_shape(self.h, which, ctypes.byref(nx), ctypes.byref(nz))
        out = np.zeros((nx.value, nz.value))
        self.L.orc_get_field(self.h, which, _dp(out))
        return out

    def solve(self, rho: np.ndarray) -> np.ndarray:
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        u = np.zeros_like(rho)
        self._check(self.L.orc_solve(self.h, _dp(rho), _dp(u)))
        return u

    def u_smooth(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros_like(u)
        self.L.orc_u_smooth(u.shape[0], u.shape[1], u.ctypes.data, out.ctypes.data)
        return out

    def grad(self, which: int, x, z):
        x = np.ascontiguousarray(x, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        gx, gz = np.zeros_like(x), np.zeros_like(x)
        self.L.orc_grad(self.h, which, len(x), _dp(x), _dp(z), _dp(gx), _dp(gz))
        return gx, gz

    def species_info(self, sp: int) -> np.ndarray:
        out = np.zeros(11)
        self.L.orc_species_info(self.h, sp, _dp(out))
        return out

    def rates(self, sp: int) -> np.ndarray:
        out = np.zeros(len(self.names))
        self.L.orc_rates(self.h, sp, _dp(out))
        return out

    def rng(self, kind: int, n: int, arg: float = 0.0) -> np.ndarray:
        out = np.zeros(n * (3 if kind >= 4 else 1))
        self.L.orc_rng(self.h, kind, n, ctypes.c_double(arg), _dp(out))
        return out

    def collisions(self, sp: int) -> int:
        """Null-collision candidates of species sp (scatter() calls)."""
        return int(self.L.orc_collisions(self.h, sp))

    def real_collisions(self, sp: int) -> int:
        """Candidates that selected an interaction (not a null collision)."""
        return int(self.L.orc_real_collisions(self.h, sp))

    def set_bfield(self, nx: int, nz: int, dx: float, dz: float, x0: float, z0: float, Br, Bz):
        """Fields::load_magnetic_field tables (src/fields.cpp:870-959) as arrays."""
        br = np.ascontiguousarray(Br, dtype=np.float64)
        bz = np.ascontiguousarray(Bz, dtype=np.float64)
        self._check(self.L.orc_set_bfield(self.h, nx, nz, ctypes.c_double(dx), ctypes.c_double(dz),
                                          ctypes.c_double(x0), ctypes.c_double(z0), _dp(br), _dp(bz)))


def to_fixed(v: np.ndarray) -> np.ndarray:
    """Grid-unit positions to the library's fixed point (cells times 2^20, round to nearest)."""
    return np.rint(np.asarray(v, dtype=np.float64) * 1048576.0).astype(np.uint32)


def deposit_fixed(nx: int, nz: int, xf: np.ndarray, zf: np.ndarray, alive=None) -> np.ndarray:
    """Fixed-point CIC deposit of the oracle (int64, units of 2^-40 per particle)
    of particles at fixed-point positions xf, zf (cells times 2^20)."""
    L = load_port()
    xg = np.ascontiguousarray(xf, dtype=np.uint32)
    zg = np.ascontiguousarray(zf, dtype=np.uint32)
    acc = np.zeros((nx, nz), dtype=np.int64)
    al = None if alive is None else np.ascontiguousarray(alive, dtype=np.uint8)
    L.orc_deposit_fixed(nx, nz, len(xg), xg.ctypes.data, zg.ctypes.data,
                        None if al is None else al.ctypes.data, acc.ctypes.data)
    return acc


# ----------------------------------------------------------------------------
# ctypes: the reference built from its own sources (only where it was built)
# ----------------------------------------------------------------------------
def ref_available() -> bool:
    return REF_SO.exists()


class Ref:
    """The reference's Pic<D> through oracle/ref/ref_harness.cpp."""

    def __init__(self, config_path, species_conf_path, outdir, seed: int = 1):
        L = ctypes.CDLL(str(REF_SO))
        L.ref_create.restype = ctypes.c_void_p
        L.ref_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint]
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_time_advance.restype = ctypes.c_double
        self.L = L
        os.makedirs(outdir, exist_ok=True)
        h = L.ref_create(str(config_path).encode(), str(species_conf_path).encode(),
                         str(outdir).encode(), seed)
        if not h:
            raise RuntimeError(L.ref_last_error().decode())
        self.h = ctypes.c_void_p(h)
        self.ns = L.ref_n_species(self.h)

    def _check(self, rc):
        if rc < 0:
            raise RuntimeError(self.L.ref_last_error().decode())
        return rc

    def __del__(self):
        try:
            self.L.ref_destroy(self.h)
        except Exception:
            pass

    def grid(self):
        dims = (ctypes.c_int * 2)()
        out = np.zeros(12)
        self.L.ref_grid(self.h, dims, _dp(out))
        return (dims[0], dims[1]), out

    def source_refresh(self, factor: int):
        self._check(self.L.ref_source_refresh(self.h, factor))

    def source_save(self, sp: int, path):
        self._check(self.L.ref_source_save(self.h, sp, str(path).encode()))

    def n_live(self, sp: int) -> int:
        return self._check(self.L.ref_n_live(self.h, sp))

    def species_info(self, sp: int):
        buf = ctypes.create_string_buffer(128)
        out = np.zeros(11)
        self.L.ref_species(self.h, sp, buf, 128, _dp(out))
        return buf.value.decode(), out

    def rates(self, sp: int) -> np.ndarray:
        out = np.zeros(self.ns)
        self.L.ref_rates(self.h, sp, _dp(out))
        return out

    def sigma_v(self, sp: int, tgt: int, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.zeros(64 * len(v))
        k = self.L.ref_sigma_v(self.h, sp, tgt, len(v), _dp(v), _dp(out))
        return out[: k * len(v)].reshape(k, len(v))

    def run_initscript(self, path):
        self._check(self.L.ref_run_initscript(self.h, str(path).encode()))

    def set_particles(self, sp: int, x, z, vx, vy, vz):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, z, vx, vy, vz)]
        self._check(self.L.ref_set_particles(self.h, sp, len(arrs[0]), *[_dp(a) for a in arrs]))

    def particles(self, sp: int) -> np.ndarray:
        n = int(self.species_info(sp)[1][8])
        out = np.zeros((max(n, 1), 8))
        self.L.ref_get_particles(self.h, sp, _dp(out))
        return out[:n]

    def save(self, sp: int, path) -> None:
        self._check(self.L.ref_save(self.h, sp, str(path).encode()))

    def load(self, sp: int, path) -> int:
        return self._check(self.L.ref_load(self.h, sp, str(path).encode()))

    def seed(self, s: int):
        self.L.ref_seed(self.h, s)

    def advance_init(self):
        self._check(self.L.ref_advance_init(self.h))

    def advance(self, n: int = 1):
        self._check(self.L.ref_advance(self.h, n))

    def time_advance(self, n: int) -> float:
        return self.L.ref_time_advance(self.h, n)

    def field(self, which: int) -> np.ndarray:
        (nx, nz), _ = self.grid()
        if which in (3, 4):
            c = ctypes.c_int()
        out = np.zeros(4 * 1024 * 1024)
        k = self.L.ref_get_field(self.h, which, _dp(out))
        if which in (0, 1, 2) or which >= 5:
            return out[:k].reshape(nx, -1) if k % nx == 0 else out[:k]
        return out[:k]

    def mask_voltage(self, x_sampl: int, z_sampl: int):
        out = np.zeros(x_sampl * z_sampl)
        self.L.ref_get_field(self.h, 3, _dp(out))
        mask = out.reshape(x_sampl, z_sampl).astype(np.int8)
        out2 = np.zeros(x_sampl * z_sampl)
        self.L.ref_get_field(self.h, 4, _dp(out2))
        return mask, out2.reshape(x_sampl, z_sampl)

    def solve(self, rho: np.ndarray) -> np.ndarray:
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        u = np.zeros_like(rho)
        self._check(self.L.ref_solve(self.h, _dp(rho), _dp(u)))
        return u

    def u_smooth(self, u: np.ndarray) -> np.ndarray:
        """Fields::u_smooth() of the reference applied to a given potential."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros_like(u)
        self._check(self.L.ref_u_smooth(self.h, _dp(u), _dp(out)))
        return out

    def grad(self, which: int, x, z):
        x = np.ascontiguousarray(x, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        gx, gz = np.zeros_like(x), np.zeros_like(x)
        self.L.ref_grad(self.h, which, len(x), _dp(x), _dp(z), _dp(gx), _dp(gz))
        return gx, gz

    def rng(self, kind: int, n: int, arg: float = 0.0) -> np.ndarray:
        out = np.zeros(n * (3 if kind >= 4 else 1))
        self.L.ref_rng(self.h, kind, n, ctypes.c_double(arg), _dp(out))
        return out
