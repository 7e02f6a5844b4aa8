#!/usr/bin/env python3
"""Benchmark of the mag2d PIC-MCC step on GB300: particle-steps/s.

Headline workload (default): the large single instance — a Penning trap on an
r-z grid of 1025 x 2049 nodes with 1e8 electron macro-particles (SoA, FP32
velocities, 32-bit fixed-point positions), B = 0.5 T, He at 1e-3 Pa with a
constant collision frequency of 1e6 s^-1 (null-collision MCC), a
self-consistent Poisson solve per step (FP32 multigrid refined in FP64 to
1e-10), particles sorted by cell every 20 steps.  One bench step = one PIC
time step (Pic::advance) of every particle.  Inputs are synthetic and seeded
(uniform in volume in r < 2 mm, 5 < z < 15 mm, Maxwellian at 1 eV).

The same JSON line embeds the other configurations under "configurations":
  penning_rz   — Penning r-z 65 x 129, 1e5 electrons, self-consistent
  multipole_xy — 22-pole RF trap 257 x 257, 1e6 ions, elastic MCC; one bench
                 step = advance(50)
  batched      — 256 independent Penning instances in one batched launch
                 sequence, against the same instances run one at a time
  adjoint      — gradients/s of the segmented Penning trap (8 voltages + B)

Timing: W untimed warm-up steps, then K timed steps, each bracketed by CUDA
events on the simulation's stream; value = live particles summed over the
timed steps / summed step time.  The large workload's particle state (2.4 GB)
is far larger than L2 (129 MB), so L2 is not flushed there; the smaller
workloads flush L2 between timed steps (a 512 MB write, then a 256 MB read).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload large|multipole|penning|batched|adjoint]

--impl reference times the CPU implementation of the step on all host cores:
the oracle port of the reference algorithm (FP64, the reference's
SHR3/ziggurat random numbers, built with the reference's -Ofast) for the
particles, and a sparse direct LU solve (SciPy SuperLU, standing in for the
reference's UMFPACK, which is not available) for the Poisson solve.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

METRIC = "PIC particle-steps/s"
UNIT = "particle-steps/s"
FLUSH_BYTES = 512 << 20
# Algorithmic bytes: a particle-step reads and writes x, z, vx, vy, vz once
# (FP32 / uint32 SoA, 2 x 5 x 4 B); a grid node of a self-consistent step adds
# an int64 deposit write and read and an FP32 potential write and read.
BYTES_PER_PARTICLE_STEP = 40
BYTES_PER_NODE_STEP = 24
# DRAM bytes per particle and launch from ncu captures (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch, divided by the particles):
#   profiles/k_push_fused_multipole_xy_1e6.md   (50 fused steps per launch)
#   profiles/k_push_penning_large_rz_2e7.md     (one step per launch)
DRAM_BYTES_PER_PARTICLE = {"multipole": 24.8, "large": 41.7}
# ncu warp instructions per 32 particle-steps of k_push_fused<0,2,0>
# (smsp__inst_executed per launch / (1e6 x 50 / 32), profiles/k_push_fused_multipole_xy_1e6.md)
FUSED_WARP_INSTR_PER_32 = 177

WORKLOADS = {
    "large": dict(particles=100_000_000, step_len=1, sort_interval=20, flush=False, species=0,
                  grid=[1025, 2049],
                  desc="penning_large: Penning trap r-z 1025x2049 grid (r 0-5 mm, z 0-20 mm), 1e8 electrons (1 eV, "
                       "uniform in r<2 mm, 5<z<15 mm), Bz 0.5 T, He 1e-3 Pa constant nu 1e6/s elastic MCC, "
                       "self-consistent (FP32 multigrid + FP64 refinement to 1e-10), dt 1 ps, sort every 20 steps"),
    "penning": dict(particles=100_000, step_len=1, sort_interval=100, flush=True, species=0, grid=[65, 129],
                    desc="penning_rz: Penning trap r-z 65x129 grid (r 0-5 mm, z 0-20 mm), end caps -10 V, ring 0 V, "
                         "Bz 1 T, 1e5 electrons 1 eV in r<2 mm, 5<z<15 mm, self-consistent (Poisson to 1e-10), "
                         "collisions off, dt 10 ps"),
    "multipole": dict(particles=1_000_000, step_len=50, sort_interval=100, flush=True, species=1, grid=[257, 257],
                      desc="multipole_xy: 22-pole RF ion trap, 257x257 x-y grid, 1e6 ions (3 amu, 0.1 eV), "
                           "He 1e-2 Pa elastic MCC, dt 2 ns"),
}


def _env_rank():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", str(r)))
    return r, w, lr


def _peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if "hbm_gbs" in d:
            return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (burst copy), of measured"
    return 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent), of fallback"


def _config(workload: str, n_gpus: int, particles: int, sort_interval: int, step_len: int) -> dict:
    w = WORKLOADS[workload]
    c = {"workload": w["desc"], "grid": w["grid"], "particles_per_gpu": particles, "sort_interval": sort_interval,
         "parallelism": f"replicas x{n_gpus}" if n_gpus > 1 else "single GPU",
         "l2": ("flushed between timed steps (512 MB write, then 256 MB read)" if w["flush"] else
                "not flushed: the particle state (24 B x particles) is far larger than L2")}
    if step_len > 1:
        c["time_steps_per_step"] = step_len
        c["step"] = (f"one advance({step_len}) call: {step_len} PIC time steps of every particle (particles are "
                     "independent without a self-consistent field, so the steps run fused in one launch)")
    else:
        c["step"] = "one advance(1) call: one PIC time step of every particle (solve, push, deposit, collisions)"
    return c


# ----------------------------------------------------------------------------
# CPU baseline: the oracle port (reference algorithm) on the host cores
def _cpu_sample(tmp: Path, workload: str, n: int, seed: int):
    """(cfg, species, inter, config path, particles, species index, loaded fields) of a per-core sample."""
    from cases import multipole_xy, penning_large, penning_rz
    from mag2d_cases import write_config

    if workload == "multipole":
        cfg, species, inter, cpath, spath, parts, loaded = multipole_xy(tmp, n=n, n_nodes=257, seed=seed)
        return cfg, species, inter, cpath, parts, 1, loaded
    if workload == "penning":
        cfg, species, inter, cpath, spath, parts = penning_rz(tmp, n=n, seed=seed)
        return cfg, species, inter, cpath, parts, 0, None
    # large: the particles of the large instance (its B, collisions, dt) on the 65 x 129 grid with the field
    # of the electrodes alone; the step's Poisson solve is timed separately on the full grid
    cfg, species, inter, cpath, spath, parts = penning_large(tmp, n=n, nr=65, nz=129, seed=seed)
    cfg = dict(cfg, selfconsistent=0)
    write_config(cfg, cpath)
    return cfg, species, inter, cpath, parts, 0, None


def _cpu_worker(args):
    """One core: the oracle port on a sample of the workload; warm untimed
    steps, then steps timed ones.  Returns (particle_steps, seconds)."""
    n, steps, seed, workload, warm = args
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np

    from mag2d_cases import Port

    with tempfile.TemporaryDirectory() as d:
        cfg, species, inter, cpath, parts, sp, loaded = _cpu_sample(Path(d), workload, n, seed)
        if loaded is not None:
            mask, volt = np.zeros((3, 3), dtype=np.int8), np.zeros((3, 3))
        else:
            from mag2d_gb300 import config_geometry

            mask, volt = config_geometry(cpath)
        port = Port(cfg, species, inter, mask, volt, seed=seed, loaded_fields=loaded, timing=True)
        port.set_particles(sp, *parts)
        port.advance_init()
        port.advance(max(warm, 1))
        live0 = port.n_live(sp)
        t = port.time_advance(steps)
        live1 = port.n_live(sp)
    return 0.5 * (live0 + live1) * steps, t


def cpu_push_rate(workload: str, sample_particles: int, sample_steps: int, warm: int = 2, cores: int | None = None):
    """All-core particle throughput of the oracle port: one independent sample per core."""
    import multiprocessing as mp

    cores = cores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(sample_particles, sample_steps, 100 + i, workload, warm) for i in range(cores)])
    wall = time.perf_counter() - t0
    ps = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    per_core = sum(r[0] / r[1] for r in res) / len(res)
    return ps / busy, per_core, cores, wall


def _superlu_worker(q, nsolves: int):
    """Sparse direct solve of the large grid's system (SciPy SuperLU, COLAMD):
    factorisation once (as the reference factorises once at start-up), then
    nsolves solves of a charge-carrying right-hand side, each followed by
    iterative refinement until the Jacobi-scaled residual is below 1e-10 of
    max|u| (at most 3 refinements).  Puts (factor_s, solve_s_mean, residual)."""
    try:
        sys.path.insert(0, str(ROOT / "tests"))
        import numpy as np
        import scipy.sparse.linalg as spl

        from cases import penning_large
        from mag2d_cases import QE, poisson_system
        from mag2d_gb300 import config_geometry

        with tempfile.TemporaryDirectory() as d:
            cfg, species, inter, cpath, spath, _ = penning_large(Path(d), make_particles=False)
            mask, volt = config_geometry(cpath)
        rho = -QE * 50 * np.random.default_rng(3).random(mask.shape)
        A, b = poisson_system(cfg, mask, volt, rho)
        diag = A.diagonal()
        t0 = time.perf_counter()
        lu = spl.splu(A.tocsc(), permc_spec="COLAMD")
        factor_s = time.perf_counter() - t0
        times, res = [], 0.0
        for _ in range(nsolves):
            t0 = time.perf_counter()
            u = lu.solve(b)
            for _ in range(3):
                r = b - A @ u
                res = np.abs(r / diag).max() / np.abs(u).max()
                if res <= 1e-10:
                    break
                u = u + lu.solve(r)
            times.append(time.perf_counter() - t0)
        q.put((factor_s, float(np.mean(times)), float(res)))
    except Exception as e:  # reported in the JSON line
        q.put(("error", repr(e), 0.0))


class SolveTimer:
    """The large grid's direct solve timed in a separate process, started early
    so that its factorisation (about a minute) overlaps the GPU measurements."""

    def __init__(self, nsolves: int = 3):
        import multiprocessing as mp

        ctx = mp.get_context("spawn")
        self.q = ctx.Queue()
        self.p = ctx.Process(target=_superlu_worker, args=(self.q, nsolves), daemon=True)
        self.p.start()

    def result(self, timeout: float = 900.0):
        r = self.q.get(timeout=timeout)
        self.p.join(timeout=10)
        if r[0] == "error":
            raise RuntimeError(f"direct solve failed: {r[1]}")
        return r


def cpu_baseline(workload: str, n_particles: int, solve_timer: SolveTimer | None = None,
                 sample_particles: int = 20_000, sample_steps: int | None = None) -> dict:
    """The CPU time of one bench step of the workload on all host cores."""
    if sample_steps is None:
        sample_steps = {"multipole": 1000, "penning": 200, "large": 200}[workload]
    rate, per_core, cores, wall = cpu_push_rate(workload, sample_particles, sample_steps)
    out = {"unit": UNIT, "cores": cores, "kind": "port", "per_core": per_core}
    if workload == "large":
        factor_s, solve_s, res = solve_timer.result()
        push_s = n_particles / rate
        step_s = push_s + solve_s
        out["value"] = n_particles / step_s
        out["ms_per_step"] = step_s * 1e3
        out["sample"] = (f"particles: {cores} independent processes x ({sample_particles} electrons x {sample_steps} "
                         f"steps) of the large instance's particle step (B 0.5 T, nu 1e6/s, dt 1 ps) with the "
                         f"electrodes' field on a 65x129 grid, FP64 oracle port built -Ofast, per-core "
                         f"{per_core:.3e} {UNIT} -> {push_s * 1e3:.1f} ms for {n_particles:.0e} particles on "
                         f"{cores} cores; Poisson: SciPy SuperLU (COLAMD) direct solve of the 1025x2049 system with "
                         f"iterative refinement to 1e-10 (UMFPACK, the reference's solver, is not available), "
                         f"{solve_s * 1e3:.0f} ms per solve on one core after a {factor_s:.0f} s factorisation "
                         f"(residual {res:.1e}); step = push + solve")
    else:
        out["value"] = rate
        out["sample"] = (f"{cores} independent processes x ({sample_particles} particles x {sample_steps} steps) of "
                         f"the same workload, FP64 oracle port built -Ofast with the reference's SHR3/ziggurat "
                         f"RNG; per-core {per_core:.3e} {UNIT}; wall {wall:.1f} s incl. set-up")
    return out


def run_reference(args) -> None:
    """--impl reference: the CPU step of the same workload on all host cores."""
    rank, world, _ = _env_rank()
    if rank != 0:
        return
    wk = args.workload
    w = WORKLOADS.get(wk)
    if w is None:
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU reference arm for workload {wk}"}))
        return
    spb = w["step_len"]
    timer = SolveTimer() if wk == "large" else None
    steps = max(args.steps, 1)
    base = cpu_baseline(wk, w["particles"], timer, sample_steps=spb * steps if wk != "large" else 10 * steps)
    v = base["value"]
    ms = base.get("ms_per_step", w["particles"] * spb / v * 1e3)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": _config(wk, args.gpus, w["particles"], w["sort_interval"], spb), "impl": "reference",
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self) -> dict:
        self.out.flush()
        rows = []
        for line in Path(self.out.name).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(r[0] for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[2 + k].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": rows[0][1], "reasons": reasons, "samples": len(rows)}


def _build(rank: int):
    import __graft_entry__

    if rank == 0 or not (ROOT / "mag2d_gb300" / "lib" / "libmag2d_gpu.so").exists():
        __graft_entry__.build()


def _make_pic(m, wk: str, tmp: Path, n: int, rank: int, local: int, sort_interval: int, push_vec: int):
    if wk == "penning":
        from cases import penning_rz

        cfg, species, inter, cpath, spath, parts = penning_rz(tmp, n=n, seed=2 + rank)
        pic = m.Pic(cpath, spath, seed=1000 + rank, device=local, capacity_hint=n, push_vec=push_vec,
                    sort_interval=sort_interval, poisson_tol=1e-10)
        pic.speclist[0].set_particles(*parts)
    elif wk == "large":
        from cases import penning_large

        cfg, species, inter, cpath, spath, _ = penning_large(tmp, n=n, make_particles=False)
        ini = tmp / "init.txt"
        ini.write_text(f"add_particles_in_cylinder ELECTRON {n} 2e-3 5e-3 15e-3\n")
        pic = m.Pic(cpath, spath, ini, seed=1000 + rank, device=local, capacity_hint=n, push_vec=push_vec,
                    sort_interval=sort_interval, poisson_tol=1e-10)
    else:
        from cases import multipole_xy

        cfg, species, inter, cpath, spath, parts, loaded = multipole_xy(tmp, n=n, n_nodes=257, seed=2 + rank)
        pic = m.Pic(cpath, spath, seed=1000 + rank, device=local, capacity_hint=n, push_vec=push_vec,
                    sort_interval=sort_interval)
        pic.speclist[1].set_particles(*parts)
    return pic, species


def measure_single(args, wk: str, rank: int = 0, world: int = 1, local: int = 0, dist=None,
                   solve_timer: SolveTimer | None = None) -> dict:
    """One instance of workload wk: device-timed steps, per-kernel times,
    roofline, end-to-end call with host arrays and the CPU baseline."""
    import numpy as np
    import torch

    import mag2d_gb300 as m

    w = WORKLOADS[wk]
    n = args.particles or w["particles"]
    L = args.step_len or w["step_len"]
    si = args.sort_interval or w["sort_interval"]
    tmp = Path(tempfile.mkdtemp(prefix=f"mag2d_bench_{wk}_{rank}_"))
    pic, species = _make_pic(m, wk, tmp, n, rank, local, si, args.push_vec)
    sp = pic.speclist[w["species"]]
    pic.advance_init()
    pic.sync()
    stream = torch.cuda.ExternalStream(pic.stream, device=local)
    if w["flush"]:
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
        clean = torch.ones(FLUSH_BYTES // 8, dtype=torch.float32, device=f"cuda:{local}")
        sink = torch.empty((), dtype=torch.float32, device=f"cuda:{local}")

    def flush_l2():
        # write 512 MB (evicts everything), then read 256 MB so that the dirty
        # lines of that write are written back before the timed step starts
        if w["flush"]:
            with torch.cuda.stream(stream):
                flush.zero_()
                torch.sum(clean, dim=0, out=sink)

    for _ in range(args.warmup):
        flush_l2()
        pic.advance(L)
    pic.sync()
    d0 = sp.diag()
    launches0 = pic.kernel_launches
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush_l2()
            starts[k].record(stream)
            pic.advance(L)
            ends[k].record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    total_s = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) * 1e-3
    d1 = sp.diag()
    launches = pic.kernel_launches - launches0
    psteps = d1["particle_steps"] - d0["particle_steps"]

    # per-kernel device time (events between the kernels of each step)
    kern = np.zeros(4)
    nk = max(3, min(args.steps, 20))
    for _ in range(nk):
        flush_l2()
        kern += np.array(pic.advance_timed(L))
    kern /= nk
    push_ms = kern[2]  # one particle launch per call: L steps fused, or a single step
    live_now = sp.diag()["n_live"]
    alg_bytes = BYTES_PER_PARTICLE_STEP * live_now * L
    achieved = alg_bytes / (push_ms * 1e-3) / 1e9
    solve_info, phases = None, None
    if wk != "multipole":
        solve_info = pic.solve_status()
        if wk == "large":
            pic.solve_phase_times()  # switches the solve's phase timers on
            pic.advance(1)
            phases = pic.solve_phase_times()

    # e2e through the C ABI with host buffers: upload the state from pinned host
    # FP64 arrays, advance e2e_steps steps, read the diagnostics back
    e2e_steps = {"large": 20, "penning": 50, "multipole": 50}[wk]
    e2e_val, n_host = 0.0, 0
    if not args.no_e2e:
        hst = sp.particles()
        host = []
        for k in ("x", "z", "vx", "vy", "vz"):
            buf = torch.empty(len(hst[k]), dtype=torch.float64).pin_memory().numpy()
            buf[:] = hst[k]
            host.append(buf)
        del hst
        n_host = len(host[0])
        best = float("inf")
        ps = 0
        for _ in range(2 if wk == "large" else 5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sp.set_particles(*host)
            pic.advance(e2e_steps)
            dd = sp.diag()
            best = min(best, time.perf_counter() - t0)
            ps = dd["n_live"] * e2e_steps
        e2e_val = ps / best
        del host

    if world > 1:
        vals = torch.tensor([total_s, psteps, e2e_val], dtype=torch.float64, device=f"cuda:{local}")
        tmax = vals[0:1].clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tot = vals[1:3].clone()
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        total_s, psteps_all, e2e_all = float(tmax), float(tot[0]), float(tot[1])
    else:
        psteps_all, e2e_all = float(psteps), float(e2e_val)
    pic.close()
    if rank != 0:
        return {}
    peak, peak_src = _peak()
    nodes = w["grid"][0] * w["grid"][1] if wk != "multipole" else 0
    step_ms = total_s / args.steps * 1e3
    line = {
        "metric": METRIC, "value": psteps_all / total_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": _config(wk, world, n, si, L),
        "clocks": clk.summary(),
        "e2e": {"value": e2e_all, "unit": UNIT,
                "h2d_bytes_per_step": int(5 * 8 * n_host * L / e2e_steps),
                "d2h_bytes_per_step": int((48 + 88 * len(species)) * L / e2e_steps),
                "note": f"e2e call = set_particles from pinned host FP64 arrays (x, z, vx, vy, vz) + "
                        f"advance({e2e_steps}) + diag read (best of {2 if wk == 'large' else 5}); bytes per bench "
                        f"step"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (DRAM_BYTES_PER_PARTICLE[wk] * live_now) if wk in DRAM_BYTES_PER_PARTICLE else None,
                     "traffic_source": {"multipole": "profiles/k_push_fused_multipole_xy_1e6.md",
                                        "large": "profiles/k_push_penning_large_rz_2e7.md"}.get(wk),
                     "kernel": ("k_push_fused<0,2,0> (50 steps per launch: gather + Boris + collision test + "
                                "background scatter + boundary)" if wk == "multipole" else
                                "k_push<1,1,1,VEC> (cylindrical gather + Boris + r map + boundary + collision test + "
                                "deposit; 4 slots per thread for 1e8 electrons, 2 for 1e5)"),
                     "alg_bytes_per_launch": alg_bytes, "bytes_per_particle_step": BYTES_PER_PARTICLE_STEP,
                     "kernel_ms": push_ms, "peak_source": peak_src},
        "kernel_ms_per_step": {"sort": kern[0] / L, "solve": kern[1] / L, "particles": kern[2] / L,
                               "collide": kern[3] / L, "per": "PIC time step"},
    }
    if nodes:
        step_bytes = BYTES_PER_PARTICLE_STEP * live_now + BYTES_PER_NODE_STEP * nodes
        line["step_roofline"] = {"achieved": step_bytes / (step_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": step_bytes / (step_ms * 1e-3) / 1e9 / peak,
                                 "alg_bytes_per_step": step_bytes,
                                 "note": "whole step: 40 B per particle + 24 B per grid node (solve, deposit)"}
        line["poisson_last_solve"] = solve_info
    if phases is not None:
        line["solve_phase_ms"] = {"start": phases["start"], "fp64_residual": phases["residual"],
                                  "down_per_level": [x for x in phases["down"] if x > 0],
                                  "coarse_block0": phases["coarse"],
                                  "up_per_level": [x for x in phases["up"] if x > 0],
                                  "faces": phases["faces"], "total": phases["total"],
                                  "note": "one solve, from the kernel's own phase timers (mag_solve_phase_times)"}
    if wk == "multipole":
        sm_mhz = line["clocks"].get("sm_mhz") or 2070.0
        ps_per_cycle = live_now * L / (push_ms * 1e-3 * sm_mhz * 1e6 * 152)
        line["issue"] = {"particle_steps_per_sm_cycle": ps_per_cycle,
                         "warp_instructions_per_32_particle_steps": FUSED_WARP_INSTR_PER_32,
                         "note": "the fused kernel is issue-bound (profiles/k_push_fused_multipole_xy_1e6.md); "
                                 "SM cycles at the sampled SM clock over 152 SMs"}
    if not args.no_cpu_baseline and world == 1:
        base = cpu_baseline(wk, n, solve_timer)
        line["cpu_baseline"] = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
    return line


def measure_batched(args, local: int = 0) -> dict:
    """256 Penning instances (uneven grids, particle counts, pressures, end caps)
    advanced by the batched path, against a sample of the same instances run
    one at a time on the plain path."""
    import numpy as np
    import torch

    import mag2d_gb300 as m
    from cases import batched_penning

    n_inst = args.instances
    tmp = Path(tempfile.mkdtemp(prefix="mag2d_batch_"))
    inst = batched_penning(tmp, n=n_inst, seed0=0)
    t0 = time.perf_counter()
    b = m.Batch([(c[3], c[4], c[5], c[6]) for c in inst], device=local, poisson_tol=1e-9)
    b.advance_init()
    setup_s = time.perf_counter() - t0
    tuning = b.tune(3)
    stream = torch.cuda.ExternalStream(b.stream, device=local)
    b.advance(args.warmup)
    b.sync()

    def live_total():
        return sum(b[i].speclist[0].diag()["particle_steps"] for i in range(len(b)))

    ps0 = live_total()
    launches0 = b.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        b.advance(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1)
    b.sync()
    psteps = live_total() - ps0
    launches = b.kernel_launches - launches0
    max_res = max(b[i].solve_status()["residual"] for i in range(len(b)))
    b.close()
    stride = max(1, n_inst // args.plain_sample)
    sample = list(range(0, n_inst, stride))
    def plain_step_ms(c, **kw):
        pic = m.Pic(c[3], c[4], c[5], seed=c[6], device=local, poisson_tol=1e-9, **kw)
        pic.advance_init()
        pic.advance(3)
        s_ = torch.cuda.ExternalStream(pic.stream, device=local)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a0.record(s_)
        pic.advance(args.plain_steps)
        a1.record(s_)
        torch.cuda.synchronize()
        res = pic.solve_status()["residual"]
        pic.close()
        return a0.elapsed_time(a1) / args.plain_steps, res

    # plain: each instance alone with the default solver (the precomputed
    # inverse on grids up to 2e4 nodes, else FP32 multigrid + FP64 refinement);
    # plain FP64: each instance alone with every multigrid level in FP64
    plain = [plain_step_ms(inst[i]) for i in sample]
    plain64 = [plain_step_ms(inst[i], direct_solve=-1, multigrid_fp64=1) for i in sample]
    plain_ms = float(np.mean([p_[0] for p_ in plain])) * n_inst  # the sweep one instance after another
    plain64_ms = float(np.mean([p_[0] for p_ in plain64])) * n_inst
    batch_step_ms = batch_ms / args.steps
    return {"metric": METRIC, "value": psteps / (batch_ms * 1e-3), "unit": UNIT, "ms_per_step": batch_step_ms,
            "steps": args.steps,
            "config": {"workload": f"batched_penning: {n_inst} Penning r-z instances, grid 65x129 or 129x257, "
                                   "1e3-1e5 electrons (log-uniform), He 1e-4-1e-1 Pa (log-uniform), end caps "
                                   "-20..-5 V, self-consistent, Poisson refined to 1e-9", "instances": n_inst},
            "clocks": clk.summary(), "gpu_launches": int(launches),
            "batched_vs_plain": {"batched_ms_per_step": batch_step_ms, "plain_ms_per_step": plain_ms,
                                 "speedup": plain_ms / batch_step_ms,
                                 "plain_fp64_multigrid_ms_per_step": plain64_ms,
                                 "speedup_vs_fp64_multigrid": plain64_ms / batch_step_ms,
                                 "plain_sample": f"{len(sample)} of {n_inst} instances (every {stride}th), "
                                                 f"{args.plain_steps} steps each, summed over the sweep",
                                 "tolerance": "every solve stops at Jacobi-scaled residual <= 1e-9 of max|u|",
                                 "max_final_poisson_residual": {
                                     "batched": max_res, "plain": max(p_[1] for p_ in plain),
                                     "plain_fp64_multigrid": max(p_[1] for p_ in plain64)}},
            "tuning": tuning, "setup_s": setup_s}


def measure_adjoint(args, local: int = 0) -> dict:
    """Gradients per second of the segmented Penning trap (8 ring segments + B):
    one adjoint run (forward with checkpoints, recomputation, reverse sweep)
    against the forward runs that central differences need."""
    import numpy as np
    import torch

    import mag2d_gb300 as m
    from cases import penning_segments

    tmp = Path(tempfile.mkdtemp(prefix="mag2d_adj_"))
    keys = [f"u_segment_{k}" for k in range(8)]
    n, steps = 100_000, args.adj_steps
    volts = np.random.default_rng(7).uniform(-15.0, -5.0, 8)
    c = penning_segments(tmp, n=n, volts=volts, Bz=1.0, tag="bench")
    pic = m.Pic(c[3], c[4], c[5], seed=c[6], poisson_tol=1e-10, device=local)
    pic.adjoint(20, keys, checkpoint=10)  # warm-up: kernels loaded, solver set up
    pic.close()
    times = []
    for _ in range(max(1, min(args.steps, 3))):
        pic = m.Pic(c[3], c[4], c[5], seed=c[6], poisson_tol=1e-10, device=local)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        info, grad = pic.adjoint(steps, keys, checkpoint=100)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        pic.close()
    pic = m.Pic(c[3], c[4], c[5], seed=c[6], poisson_tol=1e-10, device=local)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pic.advance_init()
    pic.advance(steps)
    pic.sync()
    fwd = time.perf_counter() - t0
    pic.close()
    t_adj = min(times)
    nparam = len(grad)
    return {"metric": "grads/s", "value": 1.0 / t_adj, "unit": "gradients/s", "ms_per_step": t_adj * 1e3,
            "steps": len(times),
            "config": {"workload": f"adjoint: Penning r-z 65x129, 8 ring segments (-15..-5 V) + Bz 1 T, {n} "
                                   f"electrons, {steps} steps, checkpoint every 100, collisions off, Poisson refined "
                                   "to 1e-10", "parameters": nparam},
            "gradient": {"loss": info["loss"], "d_loss_d_params": [float(x) for x in grad]},
            "forward_run_s": fwd, "central_difference_s": 2 * nparam * fwd,
            "adjoint_vs_central_difference": 2 * nparam * fwd / t_adj,
            "e2e": {"value": 1.0 / t_adj, "unit": "gradients/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 8 * nparam}}


def _sub_args(args, **kw):
    a = argparse.Namespace(**vars(args))
    a.particles = None
    a.step_len = None
    a.sort_interval = 0
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def run_ours(args) -> None:
    rank, world, local = _env_rank()
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    _build(rank)
    if dist is not None:
        dist.barrier()
    wk = args.workload
    if wk == "batched":
        line = measure_batched(args, local)
    elif wk == "adjoint":
        line = measure_adjoint(args, local)
    else:
        timer = SolveTimer() if (wk == "large" and not args.no_cpu_baseline and world == 1 and rank == 0) else None
        line = measure_single(args, wk, rank, world, local, dist, timer)
        if rank == 0 and wk == "large" and world == 1 and not args.no_configurations:
            subs = {}
            for name, fn in (("penning_rz", lambda: measure_single(_sub_args(args, steps=max(args.steps, 50)),
                                                                   "penning")),
                             ("multipole_xy", lambda: measure_single(_sub_args(args), "multipole")),
                             ("batched", lambda: measure_batched(_sub_args(args), local)),
                             ("adjoint", lambda: measure_adjoint(_sub_args(args), local))):
                try:
                    subs[name] = fn()
                except Exception as e:  # a failing sub-measurement must not hide the headline
                    subs[name] = {"error": repr(e)}
            line["configurations"] = subs
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large", choices=["large", "penning", "multipole", "batched", "adjoint"],
                    help="large: r-z 1025x2049, 1e8 electrons (default, with the other configurations embedded); "
                         "penning: r-z 65x129, 1e5 electrons; multipole: 22-pole 257x257, 1e6 ions; batched: 256 "
                         "Penning instances; adjoint: gradients/s")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configurations", action="store_true",
                    help="large workload: skip the embedded measurements of the other configurations")
    ap.add_argument("--particles", type=int, default=None, help="particles per GPU (default: the workload's own)")
    ap.add_argument("--instances", type=int, default=256, help="batched workload: instances")
    ap.add_argument("--plain-sample", type=int, default=16, help="batched workload: instances timed one at a time")
    ap.add_argument("--plain-steps", type=int, default=10, help="batched workload: steps per plain instance")
    ap.add_argument("--adj-steps", type=int, default=2000, help="adjoint workload: steps of the run")
    ap.add_argument("--push-vec", type=int, default=0, help="slots per thread of the particle kernel (0: default)")
    ap.add_argument("--sort-interval", type=int, default=0, help="steps between particle sorts (0: the workload's)")
    ap.add_argument("--step-len", type=int, default=None, help="PIC time steps per timed step (one advance() call)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
