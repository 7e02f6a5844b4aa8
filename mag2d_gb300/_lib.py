"""ctypes binding of libmag2d_gpu.so (include/mag2d_gpu.h).

The library is the only compute path: if it has not been built, loading fails
with an error that says so.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libmag2d_gpu.so"

MAG_OK = 0
MAG_U, MAG_URF, MAG_RHO, MAG_MASK, MAG_VOLTAGE, MAG_SPECIES_RHO = 0, 1, 2, 3, 4, 5


class MagOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("seed", ctypes.c_uint64), ("sort_interval", ctypes.c_int),
                ("poisson_tol", ctypes.c_double), ("poisson_max_iter", ctypes.c_int),
                ("capacity_hint", ctypes.c_int64), ("push_vec", ctypes.c_int),
                ("direct_solve", ctypes.c_int), ("max_fused_steps", ctypes.c_int),
                ("multigrid_fp64", ctypes.c_int)]


class MagSpeciesInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 64), ("type", ctypes.c_int), ("mass", ctypes.c_double),
                ("charge", ctypes.c_double), ("dt", ctypes.c_double), ("density", ctypes.c_double),
                ("temperature", ctypes.c_double), ("E_max", ctypes.c_double), ("v_max", ctypes.c_double),
                ("lifetime", ctypes.c_double), ("n_live", ctypes.c_int64), ("capacity", ctypes.c_int64),
                ("niter", ctypes.c_uint64)]


class MagDiag(ctypes.Structure):
    _fields_ = [("n_live", ctypes.c_int64), ("mean_energy_eV", ctypes.c_double),
                ("total_charge", ctypes.c_double), ("collisions", ctypes.c_int64),
                ("null_collisions", ctypes.c_int64), ("removed", ctypes.c_int64),
                ("particle_steps", ctypes.c_int64), ("niter", ctypes.c_uint64)]


class MagSolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("residual", ctypes.c_double), ("status", ctypes.c_int),
                ("levels", ctypes.c_int)]


class MagInstanceDesc(ctypes.Structure):
    _fields_ = [("config_path", ctypes.c_char_p), ("species_conf_path", ctypes.c_char_p),
                ("initscript_path", ctypes.c_char_p), ("seed", ctypes.c_uint64)]


class MagBatchTuning(ctypes.Structure):
    _fields_ = [("push_vec", ctypes.c_int), ("solve_threads", ctypes.c_int), ("sort_interval", ctypes.c_int),
                ("ms_per_step", ctypes.c_double)]


class MagAdjCfg(ctypes.Structure):
    _fields_ = [("nsteps", ctypes.c_uint64), ("checkpoint", ctypes.c_int), ("n_voltage_keys", ctypes.c_int),
                ("voltage_keys", ctypes.POINTER(ctypes.c_char_p)), ("grad_b", ctypes.c_int),
                ("w_energy", ctypes.c_double), ("w_lost", ctypes.c_double)]


class MagAdjOut(ctypes.Structure):
    _fields_ = [("loss", ctypes.c_double), ("mean_energy_eV", ctypes.c_double), ("lost_fraction", ctypes.c_double),
                ("n0", ctypes.c_int64), ("n_live", ctypes.c_int64)]


class MagError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mag2d_gpu error {code}: {msg}")
        self.code = code


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m mag2d_gb300.build` "
                           "(the GPU library is the only implementation of the step)")
    L = ctypes.CDLL(str(LIB_PATH))
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    L.mag_last_error.restype = ctypes.c_char_p
    L.mag_version.restype = ctypes.c_char_p
    L.mag_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(MagOpts),
                             ctypes.POINTER(P)]
    L.mag_destroy.argtypes = [P]
    L.mag_destroy.restype = None
    L.mag_run_initscript.argtypes = [P, ctypes.c_char_p]
    L.mag_advance_init.argtypes = [P]
    L.mag_advance_init_ex.argtypes = [P, ctypes.c_int]
    L.mag_advance.argtypes = [P, ctypes.c_uint64]
    L.mag_sync.argtypes = [P]
    L.mag_advance_timed.argtypes = [P, ctypes.c_uint64, D]
    L.mag_solve_status.argtypes = [P, ctypes.POINTER(MagSolveInfo)]
    L.mag_solve_phase_times.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    L.mag_rho_fixed_ptr.argtypes = [P, ctypes.c_int]
    L.mag_rho_fixed_ptr.restype = ctypes.c_void_p
    L.mag_set_rho_fixed.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    L.mag_dist_reset.argtypes = [P]
    L.mag_dist_sample.argtypes = [P]
    L.mag_dist_samples.argtypes = [P]
    L.mag_energy_dist.argtypes = [P, ctypes.c_int, ctypes.c_int, D, D, D]
    L.mag_get_average.argtypes = [P, ctypes.c_int, D]
    L.mag_print_distribution.argtypes = [P, ctypes.c_char_p]
    L.mag_print_field.argtypes = [P, ctypes.c_char_p]
    L.mag_print_trace.argtypes = [P, ctypes.c_char_p]
    L.mag_species_save.argtypes = [P, ctypes.c_int, ctypes.c_char_p]
    L.mag_species_load.argtypes = [P, ctypes.c_int, ctypes.c_char_p]
    L.mag_set_electrode_voltages.argtypes = [P, D, ctypes.c_int64]
    L.mag_n_live.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    L.mag_get_particles_aos.argtypes = [P, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
    L.mag_source_refresh.argtypes = [P, ctypes.c_int]
    L.mag_source_save.argtypes = [P, ctypes.c_int, ctypes.c_char_p]
    L.mag_source_load.argtypes = [P, ctypes.c_int, ctypes.c_char_p]
    L.mag_source_info.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                  ctypes.POINTER(ctypes.c_int64)]
    L.mag_particle_file_read.argtypes = [ctypes.c_char_p, ctypes.c_int64] + [D] * 7 + [
        ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.mag_particle_file_write.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int64] + [D] * 7
    L.mag_adjoint_run.argtypes = [P, ctypes.POINTER(MagAdjCfg), D, ctypes.POINTER(MagAdjOut)]
    L.mag_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(MagInstanceDesc), ctypes.POINTER(MagOpts),
                                   ctypes.POINTER(P)]
    L.mag_batch_destroy.argtypes = [P]
    L.mag_batch_destroy.restype = None
    L.mag_batch_size.argtypes = [P]
    L.mag_batch_advance_init.argtypes = [P]
    L.mag_batch_advance.argtypes = [P, ctypes.c_uint64]
    L.mag_batch_tune.argtypes = [P, ctypes.c_int, ctypes.POINTER(MagBatchTuning)]
    L.mag_batch_set_graph.argtypes = [P, ctypes.c_int]
    L.mag_batch_sync.argtypes = [P]
    L.mag_batch_instance.argtypes = [P, ctypes.c_int, ctypes.POINTER(P)]
    L.mag_batch_stream.argtypes = [P]
    L.mag_batch_stream.restype = ctypes.c_void_p
    I64 = ctypes.c_int64
    L.mag3d_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(MagOpts), ctypes.POINTER(P)]
    L.mag3d_destroy.argtypes = [P]
    L.mag3d_destroy.restype = None
    L.mag3d_grid.argtypes = [P, ctypes.POINTER(ctypes.c_int), D]
    L.mag3d_set_particles.argtypes = [P, ctypes.c_int, I64, D, D, D, D, D, D]
    L.mag3d_get_particles.argtypes = [P, ctypes.c_int, I64, D, D, D, D, D, D, ctypes.POINTER(ctypes.c_uint32),
                                      ctypes.POINTER(I64)]
    L.mag3d_advance_init.argtypes = [P]
    L.mag3d_advance.argtypes = [P, ctypes.c_uint64]
    L.mag3d_solve.argtypes = [P, D, ctypes.POINTER(MagSolveInfo)]
    L.mag3d_get_field.argtypes = [P, ctypes.c_int, D]
    L.mag3d_get_rho_fixed.argtypes = [P, ctypes.c_int, ctypes.POINTER(I64)]
    L.mag3d_diag.argtypes = [P, ctypes.c_int, ctypes.POINTER(MagDiag)]
    L.mag3d_kernel_launches.argtypes = [P]
    L.mag3d_kernel_launches.restype = I64
    L.mag_batch_kernel_launches.argtypes = [P]
    L.mag_batch_kernel_launches.restype = ctypes.c_int64
    L.mag_grid.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), D, D, D, D]
    L.mag_n_species.argtypes = [P]
    L.mag_species.argtypes = [P, ctypes.c_int, ctypes.POINTER(MagSpeciesInfo)]
    L.mag_get_field.argtypes = [P, ctypes.c_int, D]
    L.mag_get_face_field.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    L.mag_set_field.argtypes = [P, ctypes.c_int, D]
    L.mag_field_solve.argtypes = [P, ctypes.POINTER(MagSolveInfo)]
    L.mag_get_particles.argtypes = [P, ctypes.c_int, ctypes.c_int64, D, D, D, D, D,
                                    ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int64)]
    L.mag_set_particles.argtypes = [P, ctypes.c_int, ctypes.c_int64, D, D, D, D, D]
    L.mag_diag.argtypes = [P, ctypes.c_int, ctypes.POINTER(MagDiag)]
    L.mag_get_rho_fixed.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    L.mag_deposit.argtypes = [P]
    L.mag_stream.argtypes = [P]
    L.mag_stream.restype = ctypes.c_void_p
    L.mag_kernel_launches.argtypes = [P]
    L.mag_kernel_launches.restype = ctypes.c_int64
    L.mag_config_param.argtypes = [ctypes.c_char_p, ctypes.c_char_p, D]
    L.mag_config_geometry.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int8), D,
                                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.mag_config_species.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                     ctypes.POINTER(MagSpeciesInfo), D]
    _LIB = L
    return L


def check(rc: int) -> int:
    if rc < 0:
        raise MagError(rc, lib().mag_last_error().decode(errors="replace"))
    return rc
