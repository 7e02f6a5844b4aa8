"""Workload definitions shared by the GPU tests, smoke() and bench.py.

Inputs are synthetic and seeded (the reference ships no dataset):
  penning_rz   — Penning trap in r-z: 65x129 grid over r in [0, 5 mm],
                 z in [0, 20 mm] (the [-10, 10] mm trap shifted by +10 mm, the
                 reference's domain starts at 0), end caps -10 V, ring 0 V,
                 Bz = 1 T, electrons at 1 eV uniform in r < 2 mm, 5 < z < 15 mm
                 (volume-uniform, r = 2 mm sqrt(u)), dt = 1e-11 s,
                 self-consistent, collisions off.
  multipole_xy — 22-pole RF ion trap in x-y: 257x257 grid over a 10 mm square,
                 uRF = (r/r0)^11 cos(11 phi) about the centre, r0 = 5 mm,
                 V0 = 50 V, Omega = 2 pi 17 MHz, loaded through
                 electric_field_from_file; ions of 3 amu at 0.1 eV uniform in
                 r < 4 mm; He at 300 K and 1e-2 Pa; elastic collisions with
                 sigma(E) = 5e-19 m^2 (E / 0.01 eV)^-1/2 given as a RATE
                 (sigma v is constant for that sigma); dt = 2e-9 s.
  batched_penning — the batched sweep: instance i (seed i) is the Penning
                 trap on a 65x129 or 129x257 grid (50/50), N_p log-uniform in
                 [1e3, 1e5] electrons loaded by the initscript loader, He at a
                 pressure log-uniform in [1e-4, 1e-1] Pa (elastic, constant
                 sigma v = 3.6e-14 m^3/s), end caps uniform in [-20, -5] V.
  penning_segments — the adjoint case: the Penning trap with its ring wall
                 split into 8 z-segments biased by u_segment_0..7 (uniform in
                 [-15, -5] V), end caps at -25 V, Bz = 1 T, electrons at 1 eV,
                 self-consistent, collisions off.
  penning_large — the large single instance: the Penning geometry on an r-z
                 grid of 1025x2049 nodes, electrons at 1 eV, Bz = 0.5 T,
                 He at 1e-3 Pa with a constant collision frequency
                 nu = 1e6 s^-1 (elastic RATE = nu / n_He), dt = 1e-12 s
                 (omega_c dt = 0.088), self-consistent.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from mag2d_cases import AMU, KB, QE, write_config, write_field_file, write_species_conf

ME = 9.11e-31


def penning_rz(tmp: Path, n: int = 100_000, nr: int = 65, nz: int = 129, selfconsistent: int = 1,
               mpf: float = 10.0, seed: int = 1, Bz: float = 1.0, u_smooth: int = 0):
    cfg = dict(coord="CYLINDRICAL", boundary="FREE", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3,
               r_sampl=nr, z_sampl=nz, u_endcap=-10.0, u_ring=0.0, selfconsistent=selfconsistent, rf=0,
               magnetic_field_const=1, Bz=Bz, Br=0.0, Bt=0.0, do_plot=0, macroparticle_factor=mpf,
               n_particles_total=float(n), density_total=1e13, mover="ADVANCE_BORIS", u_smooth=u_smooth)
    species = [dict(name="ELECTRON", type="ELECTRON", mass=ME, charge=-QE, dt=1e-11, density=1e13,
                    temperature=11604.5)]
    cpath = write_config(cfg, tmp / "penning.txt")
    spath = write_species_conf(species, [], tmp / "penning_species.txt")
    rng = np.random.default_rng(seed)
    r = 2e-3 * np.sqrt(rng.random(n))
    z = 5e-3 + 10e-3 * rng.random(n)
    vth = np.sqrt(KB * 11604.5 / ME)
    parts = (r, z, vth * rng.standard_normal(n), vth * rng.standard_normal(n), vth * rng.standard_normal(n))
    return cfg, species, [], cpath, spath, parts


def multipole_fields(tmp: Path, n_nodes: int = 257, L: float = 10e-3, r0: float = 5e-3, order: int = 11):
    x = np.linspace(0.0, L, n_nodes)
    X, Y = np.meshgrid(x, x, indexing="ij")
    xc = L / 2
    r = np.hypot(X - xc, Y - xc)
    phi = np.arctan2(Y - xc, X - xc)
    urf = (r / r0) ** order * np.cos(order * phi)
    u = np.zeros_like(urf)
    write_field_file(tmp / "u_static.txt", x, x, u)
    write_field_file(tmp / "u_rf.txt", x, x, urf)
    dx = L / (n_nodes - 1)
    return (n_nodes, n_nodes, dx, dx, 0.0, 0.0, u, urf)


def multipole_xy(tmp: Path, n: int = 1_000_000, n_nodes: int = 257, seed: int = 2, pressure: float = 1e-2,
                 collisions: bool = True, field_files: bool = True):
    loaded = multipole_fields(tmp, n_nodes) if field_files else None
    # geometry only selects the field model here: EMPTY would short-circuit Fields::E to the
    # uniform extern_field (src/fields.hpp:126-131), any other value uses the loaded u and uRF
    cfg = dict(coord="CARTESIAN", boundary="FREE", geometry="RF_22PT", x_max=10e-3, z_max=10e-3,
               x_sampl=3, z_sampl=3, selfconsistent=0, rf=1, rf_amplitude=50.0, rf_U0=0.0,
               rf_omega=2 * np.pi * 17e6, electric_field_from_file=1,
               electric_field_static_file=str(tmp / "u_static.txt"),
               electric_field_rf_file=str(tmp / "u_rf.txt"), magnetic_field_const=1, do_plot=0,
               macroparticle_factor=1.0, mover="ADVANCE_BORIS")
    n_he = pressure / (KB * 300.0)
    mu = 3 * AMU * 6.69e-27 / (3 * AMU + 6.69e-27)
    rate = 5e-19 * np.sqrt(2 * 0.01 * QE / mu)  # sigma(E) v_rel, constant for sigma ~ E^-1/2
    species = [dict(name="HELIUM", type="NEUTRAL", mass=6.69e-27, density=float(n_he), temperature=300.0),
               dict(name="ION", type="ION", mass=3 * AMU, charge=QE, dt=2e-9, density=1e10,
                    temperature=1160.45)]
    inter = [dict(name="ION_He_ELASTIC", type="ELASTIC", primary="ION", secondary="HELIUM",
                  rate=float(rate))] if collisions else []
    cpath = write_config(cfg, tmp / "multipole.txt")
    spath = write_species_conf(species, inter, tmp / "multipole_species.txt")
    rng = np.random.default_rng(seed)
    rr = 4e-3 * np.sqrt(rng.random(n))
    ph = 2 * np.pi * rng.random(n)
    vth = np.sqrt(KB * 1160.45 / (3 * AMU))
    parts = (5e-3 + rr * np.cos(ph), 5e-3 + rr * np.sin(ph), vth * rng.standard_normal(n),
             vth * rng.standard_normal(n), vth * rng.standard_normal(n))
    return cfg, species, inter, cpath, spath, parts, loaded


def penning_large(tmp: Path, n: int = 100_000_000, nr: int = 1025, nz: int = 2049, mpf: float = 1.0,
                  seed: int = 1, nu: float = 1e6, pressure: float = 1e-3, make_particles: bool = True):
    """Large single instance: r-z 1025x2049, B = 0.5 T, constant-nu electron-He collisions."""
    cfg = dict(coord="CYLINDRICAL", boundary="FREE", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3,
               r_sampl=nr, z_sampl=nz, u_endcap=-10.0, u_ring=0.0, selfconsistent=1, rf=0,
               magnetic_field_const=1, Bz=0.5, Br=0.0, Bt=0.0, do_plot=0, macroparticle_factor=mpf,
               n_particles_total=float(n), density_total=1e13, mover="ADVANCE_BORIS")
    n_he = pressure / (KB * 300.0)
    species = [dict(name="ELECTRON", type="ELECTRON", mass=ME, charge=-QE, dt=1e-12, density=1e13,
                    temperature=11604.5),
               dict(name="HE", type="NEUTRAL", mass=4 * AMU, density=n_he, temperature=300.0)]
    inter = [dict(name="e_he", type="ELASTIC", primary="ELECTRON", secondary="HE", rate=nu / n_he)]
    cpath = write_config(cfg, tmp / "penning_large.txt")
    spath = write_species_conf(species, inter, tmp / "penning_large_species.txt")
    parts = None
    if make_particles:
        rng = np.random.default_rng(seed)
        r = 2e-3 * np.sqrt(rng.random(n))
        z = 5e-3 + 10e-3 * rng.random(n)
        vth = np.sqrt(KB * 11604.5 / ME)
        parts = (r, z, vth * rng.standard_normal(n), vth * rng.standard_normal(n), vth * rng.standard_normal(n))
    return cfg, species, inter, cpath, spath, parts


def batched_penning(tmp: Path, n: int = 256, seed0: int = 0, np_range=(1e3, 1e5), grids=((65, 129), (129, 257)),
                    pressure_range=(1e-4, 1e-1), endcap_range=(-20.0, -5.0)):
    """The batched sweep: list of (cfg, species, inter, config path, species path, initscript path, seed)."""
    out = []
    for i in range(n):
        seed = seed0 + i
        rng = np.random.default_rng(10_000 + seed)
        nr, nz = grids[int(rng.integers(0, len(grids)))]
        npart = int(round(np.exp(rng.uniform(np.log(np_range[0]), np.log(np_range[1])))))
        pressure = float(np.exp(rng.uniform(np.log(pressure_range[0]), np.log(pressure_range[1]))))
        u_end = float(rng.uniform(*endcap_range))
        d = tmp / f"inst{i:04d}"
        d.mkdir(parents=True, exist_ok=True)
        cfg = dict(coord="CYLINDRICAL", boundary="FREE", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3,
                   r_sampl=nr, z_sampl=nz, u_endcap=u_end, u_ring=0.0, selfconsistent=1, rf=0,
                   magnetic_field_const=1, Bz=1.0, Br=0.0, Bt=0.0, do_plot=0, macroparticle_factor=10.0,
                   n_particles_total=float(npart), density_total=1e13, mover="ADVANCE_BORIS")
        n_he = pressure / (KB * 300.0)
        species = [dict(name="ELECTRON", type="ELECTRON", mass=ME, charge=-QE, dt=1e-11, density=1e13,
                        temperature=11604.5),
                   dict(name="HE", type="NEUTRAL", mass=4 * AMU, density=n_he, temperature=300.0)]
        inter = [dict(name="e_he", type="ELASTIC", primary="ELECTRON", secondary="HE", rate=3.6e-14)]
        cpath = write_config(cfg, d / "config.txt")
        spath = write_species_conf(species, inter, d / "species_conf.txt")
        ipath = d / "initscript.txt"
        ipath.write_text(f"add_particles_in_cylinder ELECTRON {npart} 2e-3 5e-3 15e-3\n")
        out.append((cfg, species, inter, cpath, spath, ipath, seed))
    return out


def penning_segments(tmp: Path, n: int = 100_000, volts=None, Bz: float = 1.0, seed: int = 1, endcap: float = -25.0,
                     nr: int = 65, nz: int = 129, tag: str = ""):
    """Adjoint case: 8 ring segments (u_segment_k), particles loaded by the initscript loader."""
    if volts is None:
        volts = np.random.default_rng(100 + seed).uniform(-15.0, -5.0, 8)
    cfg = dict(coord="CYLINDRICAL", boundary="FREE", geometry="PENNING_ENDCAP", r_max=5e-3, z_max=20e-3,
               r_sampl=nr, z_sampl=nz, u_endcap=endcap, u_ring=0.0, ring_segments=8, selfconsistent=1, rf=0,
               magnetic_field_const=1, Bz=float(Bz), Br=0.0, Bt=0.0, do_plot=0, macroparticle_factor=10.0,
               n_particles_total=float(n), density_total=1e13, mover="ADVANCE_BORIS")
    for k, v in enumerate(volts):
        cfg[f"u_segment_{k}"] = float(v)
    species = [dict(name="ELECTRON", type="ELECTRON", mass=ME, charge=-QE, dt=1e-11, density=1e13,
                    temperature=11604.5)]
    d = tmp / f"seg{tag}"
    d.mkdir(parents=True, exist_ok=True)
    cpath = write_config(cfg, d / "config.txt")
    spath = write_species_conf(species, [], d / "species_conf.txt")
    ipath = d / "initscript.txt"
    ipath.write_text(f"add_particles_in_cylinder ELECTRON {n} 2e-3 5e-3 15e-3\n")
    return cfg, species, [], cpath, spath, ipath, seed
