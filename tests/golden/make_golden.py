#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own sources, compiled by `make -C oracle ref` into
oracle/_ref/libmag2d_ref.so (only possible where the reference tree is
present), and stores inputs and outputs as small .npz files:

  rng.npz              SHR3/ziggurat draws (uni, rnor, rexp, iuni, rot, deflect)
  step_<case>.npz      particle states after N reference time steps
  solve_<case>.npz     Fields::boundary_solve of a given rho
  u_smooth.npz         Fields::u_smooth of given potentials (the step case
                       step_penning_sc_smooth.npz runs it inside Pic::advance)
  geometry.npz         t_grid mask and voltage of every reference geometry
  params.npz           derived Param values of the reference's config files
  species.npz          parsed species, rates and lifetimes of its species_conf files
  particles_ref.dat    a particle file written by BaseSpecies::save, with its
  particles.npz        inputs, and the particles BaseSpecies::load makes of a
                       file holding particles outside the domain

The CPU tests replay the same inputs through the oracle port (bit-exact) and
through the product's host-side parser and geometry builder.
Usage: python tests/golden/make_golden.py [reference tree]   (or MAG2D_REFERENCE=...)
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from mag2d_cases import AMU, KB, QE, Ref, full_config, write_config, write_field_file, write_species_conf  # noqa: E402

import os  # noqa: E402

# the reference tree: MAG2D_REFERENCE or the first argument overrides the default location
REF_ROOT = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MAG2D_REFERENCE", "/root/reference"))
TMP = Path(tempfile.mkdtemp(prefix="golden_"))


def save(name: str, **arrays):
    np.savez_compressed(HERE / name, **arrays)
    print("wrote", name, (HERE / name).stat().st_size, "bytes")


def meta(**kw) -> np.ndarray:
    return np.array(json.dumps(kw))


# ---------------------------------------------------------------------------
def gen_rng():
    cfg = dict(coord="CARTESIAN", geometry="EMPTY", x_sampl=5, z_sampl=5, selfconsistent=0, rf=0, do_plot=0)
    sp = [dict(name="E", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, temperature=1e4)]
    ref = Ref(write_config(cfg, TMP / "rng.txt"), write_species_conf(sp, [], TMP / "rng_s.txt"), TMP / "o", 1)
    out = {}
    for seed in (1, 1234, 4242):
        ref.seed(seed)
        out[f"uni_{seed}"] = ref.rng(0, 1000)
        out[f"rnor_{seed}"] = ref.rng(1, 4000)
        out[f"rexp_{seed}"] = ref.rng(2, 4000)
        out[f"iuni_{seed}"] = ref.rng(3, 500)
        out[f"rot_{seed}"] = ref.rng(4, 500)
        out[f"deflect_{seed}"] = ref.rng(5, 500, 0.75 * np.pi)
    save("rng.npz", **out)


# ---------------------------------------------------------------------------
def run_step_case(name, cfg, species, inter, nsteps, snaps, seed, setp=None, initscript=None, fields=None):
    d = TMP / name
    d.mkdir(exist_ok=True)
    if fields is not None:
        nx, nz, dx, dz, u, urf = fields
        x = np.arange(nx) * dx
        z = np.arange(nz) * dz
        write_field_file(d / "u.txt", x, z, u)
        write_field_file(d / "urf.txt", x, z, urf)
        cfg = dict(cfg, electric_field_static_file=str(d / "u.txt"), electric_field_rf_file=str(d / "urf.txt"))
    cp = write_config(cfg, d / "config.txt")
    sp = write_species_conf(species, inter, d / "species.txt")
    ref = Ref(cp, sp, d / "out", seed)
    c = full_config(cfg)
    mask, volt = ref.mask_voltage(int(float(c["x_sampl"])), int(float(c["z_sampl"])))
    arrays = {"mask": mask, "voltage": volt}
    if setp:
        for s, parts in setp.items():
            ref.set_particles(s, *parts)
            arrays[f"init_{s}"] = np.array(parts)
    if initscript:
        (d / "init.txt").write_text(initscript)
        ref.run_initscript(d / "init.txt")
    ref.advance_init()
    for s in range(len(species)):
        arrays[f"p_init_{s}"] = ref.particles(s)
    done = 0
    for k in snaps:
        ref.advance(k - done)
        done = k
        for s in range(len(species)):
            arrays[f"p_{k}_{s}"] = ref.particles(s)
    arrays["u"] = ref.field(0)
    arrays["rho"] = ref.field(2)
    if fields is not None:
        arrays["f_u"], arrays["f_urf"] = fields[4], fields[5]
        arrays["f_grid"] = np.array(fields[:4], dtype=float)
    arrays["meta"] = meta(cfg={k: v for k, v in cfg.items() if k not in ("electric_field_static_file", "electric_field_rf_file")},
                          species=species, inter=inter,
                          nsteps=nsteps, snaps=list(snaps), seed=seed, initscript=initscript or "",
                          has_fields=fields is not None)
    save(f"step_{name}.npz", **arrays)


def gen_steps():
    # Cartesian RF 22-pole (geometry solve of uRF), ELASTIC table + LANGEVIN, initscript loaders
    cfg = dict(coord="CARTESIAN", boundary="FREE", geometry="RF_22PT", x_max=2e-2, z_max=2e-2, x_sampl=81,
               z_sampl=81, selfconsistent=0, rf=1, rf_amplitude=40.0, rf_freq=17e6, extern_field=0.0,
               magnetic_field_const=1, do_plot=0, n_particles_total=1e4, density_total=1e11,
               macroparticle_factor=1.0)
    sp = [dict(name="HELIUM", type="NEUTRAL", mass=6.69e-27, density=2e21, temperature=300.0),
          dict(name="IONS", type="ION", mass=3 * AMU, charge=QE, dt=2e-9, density=1e10, temperature=1160.45,
               emax=2.0)]
    inter = [dict(name="el", type="ELASTIC", primary="IONS", secondary="HELIUM",
                  table=[(0.0, 8e-19), (0.01, 5e-19), (0.1, 1.6e-19), (1.0, 5e-20), (10.0, 1.6e-20)]),
             dict(name="lang", type="LANGEVIN", primary="IONS", secondary="HELIUM", rate=1e-15, cutoff=3.0)]
    run_step_case("rf22_mcc", cfg, sp, inter, 100, [50, 100], 7,
                  initscript="add_particles_on_disk IONS 300 1e-2 1e-2 3e-3\nadd_particles_everywhere IONS 50\n"
                             "add_particles_bessel IONS 40 1e-2 1e-2 2e-3\n"
                             "add_tracked_particle IONS 1e-2 1e-2 100 10 0\n")
    # cylindrical self-consistent Penning-Malmberg trap (PENNING_SIMPLE), B = 0.03 T
    rng = np.random.default_rng(3)
    n = 400
    r = 2e-3 * np.sqrt(rng.random(n))
    z = 3.5e-2 + 5e-3 * (rng.random(n) - 0.5)
    vth = np.sqrt(KB * 11604.5 / 9.11e-31)
    parts = (r, z, vth * rng.standard_normal(n), vth * rng.standard_normal(n), vth * rng.standard_normal(n))
    cfg = dict(coord="CYLINDRICAL", boundary="FREE", geometry="PENNING_SIMPLE", r_max=1.2e-2, z_max=7.5e-2,
               r_sampl=25, z_sampl=76, selfconsistent=1, rf=0, magnetic_field_const=1, Bz=0.03, do_plot=0,
               macroparticle_factor=2e4, n_particles_total=4e5)
    sp = [dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, density=1e15,
               temperature=11604.5)]
    run_step_case("penning_sc", cfg, sp, [], 60, [30, 60], 5, setp={0: parts})
    # periodic EMPTY box, electron-He ELASTIC + 2 SUPERELASTIC tables (species_conf_MCC.txt)
    from mag2d_cases import Port  # noqa: F401
    txt = (REF_ROOT / "species_conf_MCC.txt").read_text()
    inter = []
    for b in txt.split("INTERACTION")[1:]:
        import re
        name = re.search(r"NAME (\S+)", b).group(1)
        typ = re.search(r"TYPE (\S+)", b).group(1)
        de = re.search(r"\bDE (\S+)", b)
        tab = b.split("CROSS_SECTION")[1].split("END_")[0]
        rows = [tuple(map(float, line.split())) for line in tab.strip().splitlines()
                if line.strip() and not line.strip().startswith("#")]
        it = dict(name=name, type=typ, primary="ELECTRON", secondary="HELIUM", table=rows)
        if de:
            it["DE"] = float(de.group(1))
        inter.append(it)
    cfg = dict(coord="CARTESIAN", boundary="PERIODIC", geometry="EMPTY", x_max=2e-2, z_max=2e-2, x_sampl=11,
               z_sampl=11, selfconsistent=0, rf=0, extern_field=1000.0, do_plot=0)
    sp = [dict(name="HELIUM", type="NEUTRAL", mass=6.69e-27, density=1e23, temperature=300.0),
          dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-1.602189e-19, dt=1e-11, density=1e17,
               temperature=10000.0, emax=30.0)]
    run_step_case("empty_superelastic", cfg, sp, inter, 150, [75, 150], 11,
                  initscript="add_particles_on_disk ELECTRON 1500 1e-2 1e-2 1e-3\n")
    # the same electron swarm under the event-driven ADVANCE_MULTICOLL mover
    run_step_case("multicoll_eedf", dict(cfg, mover="ADVANCE_MULTICOLL"), sp, inter, 60, [30, 60], 17,
                  initscript="add_particles_everywhere ELECTRON 1000\n")
    # charge exchange with neutrals and Coulomb collisions between two ion species
    cfg = dict(coord="CARTESIAN", boundary="PERIODIC", geometry="EMPTY", x_max=1e-2, z_max=1e-2, x_sampl=9,
               z_sampl=9, selfconsistent=0, rf=0, extern_field=50.0, do_plot=0)
    sp = [dict(name="AR", type="NEUTRAL", mass=40 * AMU, density=5e21, temperature=300.0),
          dict(name="ARP", type="ION", mass=40 * AMU, charge=QE, dt=1e-8, density=1e16, temperature=3000.0,
               emax=5.0),
          dict(name="HEP", type="ION", mass=4 * AMU, charge=QE, dt=1e-8, density=1e16, temperature=3000.0,
               emax=5.0)]
    inter = [dict(name="cx", type="CX", primary="ARP", secondary="AR", rate=5e-16),
             dict(name="coul", type="COULOMB", primary="ARP", secondary="HEP"),
             dict(name="hel", type="ELASTIC", primary="HEP", secondary="AR", rate=3e-16)]
    run_step_case("cx_coulomb", cfg, sp, inter, 80, [40, 80], 21,
                  initscript="add_particles_everywhere ARP 400\nadd_particles_everywhere HEP 300\n")
    # RF multipole from field tables (electric_field_from_file), elastic RATE
    L, nn = 10e-3, 65
    xg = np.linspace(0, L, nn)
    X, Y = np.meshgrid(xg, xg, indexing="ij")
    rr = np.hypot(X - L / 2, Y - L / 2)
    ph = np.arctan2(Y - L / 2, X - L / 2)
    urf = (rr / 5e-3) ** 11 * np.cos(11 * ph)
    u = 0.2 * ((X - L / 2) ** 2 - (Y - L / 2) ** 2) / (L / 2) ** 2
    cfg = dict(coord="CARTESIAN", boundary="FREE", geometry="RF_22PT", x_max=L, z_max=L, x_sampl=3, z_sampl=3,
               selfconsistent=0, rf=1, rf_amplitude=50.0, rf_U0=0.5, rf_omega=2 * np.pi * 17e6,
               electric_field_from_file=1, magnetic_field_const=1, do_plot=0)
    sp = [dict(name="HELIUM", type="NEUTRAL", mass=6.69e-27, density=2.4e21, temperature=300.0),
          dict(name="ION", type="ION", mass=3 * AMU, charge=QE, dt=2e-9, density=1e10, temperature=1160.45)]
    inter = [dict(name="el", type="ELASTIC", primary="ION", secondary="HELIUM", rate=5.3e-16)]
    rng = np.random.default_rng(9)
    n = 500
    r = 4e-3 * np.sqrt(rng.random(n))
    a = 2 * np.pi * rng.random(n)
    vth = np.sqrt(KB * 1160.45 / (3 * AMU))
    parts = (L / 2 + r * np.cos(a), L / 2 + r * np.sin(a), vth * rng.standard_normal(n),
             vth * rng.standard_normal(n), vth * rng.standard_normal(n))
    run_step_case("file_multipole", cfg, sp, inter, 120, [60, 120], 13, setp={1: parts},
                  fields=(nn, nn, L / (nn - 1), L / (nn - 1), u, urf))


# ---------------------------------------------------------------------------
def gen_solves():
    rng = np.random.default_rng(17)
    cases = {
        "penning_cyl": dict(coord="CYLINDRICAL", geometry="PENNING", r_max=1.2e-2, z_max=7.5e-2, r_sampl=41,
                            z_sampl=81),
        "rf8pt_cart": dict(coord="CARTESIAN", geometry="RF_8PT", x_max=2e-2, z_max=2e-2, x_sampl=61, z_sampl=61,
                           extern_field=200.0),
    }
    for name, g in cases.items():
        cfg = dict(selfconsistent=1, rf=0, do_plot=0, macroparticle_factor=1e3, **g)
        sp = [dict(name="E", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, temperature=1e4, density=1e13)]
        ref = Ref(write_config(cfg, TMP / f"{name}.txt"), write_species_conf(sp, [], TMP / f"{name}_s.txt"),
                  TMP / "o", 1)
        c = full_config(cfg)
        nx, nz = int(float(c["x_sampl"])), int(float(c["z_sampl"]))
        mask, volt = ref.mask_voltage(nx, nz)
        rho = -QE * 50 * rng.random((nx, nz))
        u = ref.solve(rho)
        save(f"solve_{name}.npz", mask=mask, voltage=volt, rho=rho, u=u, meta=meta(cfg=cfg, species=sp))


# ---------------------------------------------------------------------------
GEOMS = {
    "EMPTY": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=41, z_sampl=41, extern_field=250.0),
    "PROBE": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=81, z_sampl=81, probe_radius=1.5e-3,
                  u_probe=-7.0, extern_field=120.0),
    "RF_22PT": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=101, z_sampl=101),
    "RF_8PT": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=81, z_sampl=81, extern_field=90.0),
    "RF_HAITRAP": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=201, z_sampl=201, extern_field=100.0),
    "RF_QUAD": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=81, z_sampl=81),
    "TUBE": dict(coord="CARTESIAN", x_max=2e-2, z_max=2e-2, x_sampl=61, z_sampl=61, probe_radius=8e-3),
    "MAC": dict(coord="CYLINDRICAL", r_max=5e-2, z_max=4.2e-1, r_sampl=41, z_sampl=211, u_probe=-3.0),
    "PENNING": dict(coord="CYLINDRICAL", r_max=1.2e-2, z_max=7.5e-2, r_sampl=61, z_sampl=151),
    "PENNING_SIMPLE": dict(coord="CYLINDRICAL", r_max=1.2e-2, z_max=7.5e-2, r_sampl=49, z_sampl=151),
}


def gen_geometry():
    out = {}
    cfgs = {}
    for g, kw in GEOMS.items():
        cfg = dict(geometry=g, selfconsistent=0, rf=0, do_plot=0, **kw)
        sp = [dict(name="E", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, temperature=1e4)]
        ref = Ref(write_config(cfg, TMP / f"g_{g}.txt"), write_species_conf(sp, [], TMP / f"g_{g}_s.txt"),
                  TMP / "o", 1)
        c = full_config(cfg)
        mask, volt = ref.mask_voltage(int(float(c["x_sampl"])), int(float(c["z_sampl"])))
        out[f"mask_{g}"] = mask
        out[f"voltage_{g}"] = np.where(np.isin(mask, (0, 1)), volt, 0.0)
        cfgs[g] = cfg
    out["meta"] = meta(cfgs=cfgs)
    save("geometry.npz", **out)


def gen_params_species():
    keys = ["dx", "dz", "x_min", "z_min", "x_max", "z_max", "V", "dV", "dy", "macroparticle_factor"]
    out, names = {}, []
    for cf in ["config.txt", "config_MCC.txt", "config_test_MCC.txt", "config_haitrap.txt", "config_CRR.txt"]:
        src = (REF_ROOT / cf).read_text().replace("do_plot = 1", "do_plot = 0")
        p = TMP / cf
        p.write_text(src)
        try:
            ref = Ref(p, REF_ROOT / "species_conf_MCC.txt", TMP / "o", 1)
        except RuntimeError as e:
            print("skip", cf, e)
            continue
        _, vals = ref.grid()
        out[f"param_{cf}"] = vals[:10]
        out[f"text_{cf}"] = np.array(src)
        names.append(cf)
    out["param_keys"] = np.array(keys)
    out["param_configs"] = np.array(names)
    # species_conf files: parsed values, rates and lifetimes
    cfg = dict(coord="CARTESIAN", geometry="EMPTY", x_sampl=5, z_sampl=5, selfconsistent=0, rf=0, do_plot=0)
    cp = write_config(cfg, TMP / "sp_cfg.txt")
    for scf in ["species_conf.txt", "species_conf_MCC.txt"]:
        ref = Ref(cp, REF_ROOT / scf, TMP / "o", 1)
        rows, rates = [], []
        for s in range(ref.ns):
            name, info = ref.species_info(s)
            rows.append(info[:8])
            rates.append(ref.rates(s))
        out[f"species_{scf}"] = np.array(rows)
        out[f"rates_{scf}"] = np.array(rates)
        out[f"text_{scf}"] = np.array((REF_ROOT / scf).read_text())
        v = np.linspace(0, 3e6, 64)
        sv = []
        for s in range(ref.ns):
            for t in range(ref.ns):
                tab = ref.sigma_v(s, t, v)
                if tab.size:
                    sv.append((s, t, tab))
        out[f"sigmav_{scf}"] = np.array([json.dumps([(s, t, x.tolist()) for s, t, x in sv])])
    save("params_species.npz", **out)


def gen_particle_file():
    """BaseSpecies::save of known particles, and BaseSpecies::load of a file
    with particles outside the domain (they are redrawn inside it)."""
    cfg = dict(coord="CARTESIAN", geometry="EMPTY", x_max=1e-2, z_max=2e-2, x_sampl=9, z_sampl=17,
               selfconsistent=0, rf=0, do_plot=0)
    cp = write_config(cfg, TMP / "pf_cfg.txt")
    sp = write_species_conf([dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11,
                                  temperature=11604.5)], [], TMP / "pf_sp.txt")
    rng = np.random.default_rng(44)
    n = 50
    x = rng.uniform(0, 1e-2, n)
    z = rng.uniform(0, 2e-2, n)
    v = rng.normal(0, 5e5, (3, n))
    ref = Ref(cp, sp, TMP / "o", 1)
    ref.set_particles(0, x, z, v[0], v[1], v[2])
    ref.save(0, HERE / "particles_ref.dat")
    # a file whose particles 0, 7, 19 lie outside the domain
    xo, zo = x.copy(), z.copy()
    xo[0], zo[7], xo[19], zo[19] = -1e-3, 3e-2, 2e-2, -5e-3
    ref2 = Ref(cp, sp, TMP / "o", 1)
    ref2.set_particles(0, xo, zo, v[0], v[1], v[2])
    ref2.save(0, TMP / "oob.dat")
    ref3 = Ref(cp, sp, TMP / "o", 1)
    ref3.load(0, TMP / "oob.dat")
    loaded = ref3.particles(0)
    save("particles.npz", x=x, z=z, vx=v[0], vy=v[1], vz=v[2], x_oob=xo, z_oob=zo, loaded=loaded,
         meta=meta(cfg=cfg))


def gen_source():
    """Species<CARTESIAN>::source5_refresh / source of the reference: the box
    file after the refresh (source5_save) and the live particle count of the
    domain every 10 steps while the boundary inflow fills it."""
    cfg = dict(coord="CARTESIAN", geometry="EMPTY", boundary="FREE", x_max=1e-2, z_max=1e-2, x_sampl=21,
               z_sampl=21, selfconsistent=0, rf=0, do_plot=0, use_source=1, src_fact=10, extern_field=0.0,
               magnetic_field_const=1, Bz=0.0, Br=0.0, Bt=0.0, n_particles_total=1e5, density_total=1e13,
               mover="ADVANCE_BORIS")
    species = [dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-10, density=1e12,
                    temperature=11604.5)]
    cp = write_config(cfg, TMP / "src_cfg.txt")
    sp = write_species_conf(species, [], TMP / "src_sp.txt")
    ref = Ref(cp, sp, TMP / "o", 7)
    ref.set_particles(0, np.array([5e-3]), np.array([5e-3]), np.zeros(1), np.zeros(1), np.zeros(1))
    ref.advance_init()
    ref.source_refresh(cfg["src_fact"])
    ref.source_save(0, HERE / "source_ref.dat")
    steps, live = [0], [ref.n_live(0)]
    for k in range(30):
        ref.advance(10)
        steps.append(10 * (k + 1))
        live.append(ref.n_live(0))
    save("source.npz", steps=np.array(steps), live=np.array(live), meta=meta(cfg=cfg, species=species))


def gen_field3d():
    """Field3D::accumulate / interpolate / grad of the reference's header
    (oracle/ref/field3d_harness.cpp) at random points of a 9 x 7 x 11 grid."""
    import ctypes

    L = ctypes.CDLL(str(HERE.parents[1] / "oracle" / "_ref" / "libmag3d_ref.so"))
    rng = np.random.default_rng(33)
    nx, ny, nz = 9, 7, 11
    d = (1.0e-3, 1.5e-3, 0.8e-3)
    n = 60
    # within (n - 1.5) cells of the origin: nearer the far face the
    # reference's grad_component reads one node past its arrays (with weight 0)
    pts = [rng.uniform(0, (m - 1.5) * h, n) for m, h in zip((nx, ny, nz), d)]
    pts[0][:3] = [0.0, 2 * d[0], 0.3 * d[0]]  # on the origin plane, a node plane, the clamped half cell
    pts[2][3:6] = [0.0, 5 * d[2], 0.2 * d[2]]
    charge = rng.uniform(-2e-19, 2e-19, n)
    u = rng.normal(0, 1, (nx, ny, nz))
    rho = np.zeros(nx * ny * nz)
    interp = np.zeros(n)
    grad = np.zeros(3 * n)
    dp = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    L.ref3d_field(nx, ny, nz, ctypes.c_double(d[0]), ctypes.c_double(d[1]), ctypes.c_double(d[2]), n,
                  dp(pts[0]), dp(pts[1]), dp(pts[2]), dp(charge), dp(rho), dp(u), dp(interp), dp(grad))
    save("field3d.npz", shape=np.array([nx, ny, nz]), d=np.array(d), x=pts[0], y=pts[1], z=pts[2], charge=charge,
         u=u, rho=rho.reshape(nx, ny, nz), interp=interp, grad=grad.reshape(n, 3))


# ---------------------------------------------------------------------------
def gen_smooth():
    """Fields::u_smooth on random potentials of a cylindrical and a Cartesian
    grid, and the self-consistent Penning step case with u_smooth = 1."""
    out = {}
    for tag, cfg in (("cyl", dict(coord="CYLINDRICAL", geometry="PENNING_SIMPLE", r_max=1.2e-2, z_max=7.5e-2,
                                  r_sampl=25, z_sampl=76)),
                     ("cart", dict(coord="CARTESIAN", geometry="EMPTY", x_max=2e-2, z_max=1e-2, x_sampl=33,
                                   z_sampl=17))):
        cfg = dict(cfg, boundary="FREE", selfconsistent=1, rf=0, magnetic_field_const=1, do_plot=0, u_smooth=1)
        sp = [dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, density=1e15,
                   temperature=11604.5)]
        d = TMP / f"smooth_{tag}"
        d.mkdir(exist_ok=True)
        ref = Ref(write_config(cfg, d / "config.txt"), write_species_conf(sp, [], d / "species.txt"), d / "out", 1)
        c = full_config(cfg)
        shape = (int(float(c["x_sampl"])), int(float(c["z_sampl"])))
        u = np.random.default_rng(41 if tag == "cyl" else 43).normal(0.0, 1.0, shape)
        out[f"u_{tag}"] = u
        out[f"smooth_{tag}"] = ref.u_smooth(u)
    save("u_smooth.npz", **out)
    rng = np.random.default_rng(3)
    n = 400
    r = 2e-3 * np.sqrt(rng.random(n))
    z = 3.5e-2 + 5e-3 * (rng.random(n) - 0.5)
    vth = np.sqrt(KB * 11604.5 / 9.11e-31)
    parts = (r, z, vth * rng.standard_normal(n), vth * rng.standard_normal(n), vth * rng.standard_normal(n))
    cfg = dict(coord="CYLINDRICAL", boundary="FREE", geometry="PENNING_SIMPLE", r_max=1.2e-2, z_max=7.5e-2,
               r_sampl=25, z_sampl=76, selfconsistent=1, rf=0, magnetic_field_const=1, Bz=0.03, do_plot=0,
               macroparticle_factor=2e4, n_particles_total=4e5, u_smooth=1)
    sp = [dict(name="ELECTRON", type="ELECTRON", mass=9.11e-31, charge=-QE, dt=1e-11, density=1e15,
               temperature=11604.5)]
    run_step_case("penning_sc_smooth", cfg, sp, [], 60, [30, 60], 5, setp={0: parts})


if __name__ == "__main__":
    import sys

    cases = {"rng": gen_rng, "steps": gen_steps, "solves": gen_solves, "geometry": gen_geometry,
             "params_species": gen_params_species, "particle_file": gen_particle_file, "source": gen_source,
             "field3d": gen_field3d, "smooth": gen_smooth}
    for name in (sys.argv[1:] or list(cases)):
        cases[name]()
