"""mag2d_gb300 — GB300 (sm_103a) implementation of the mag2d PIC-MCC time step.

The step runs in hand-written CUDA kernels inside libmag2d_gpu.so, reached
through its C ABI (include/mag2d_gpu.h); this package is the Python side of
that boundary, shaped like the reference's Pic / Fields / Species classes.
"""
from .pic import (Batch, Fields, Pic, Pic3D, Species, config_geometry, config_param, config_species,  # noqa: F401
                  read_particle_file, write_particle_file)

__all__ = ["Pic", "Pic3D", "Batch", "Fields", "Species", "config_param", "config_geometry", "config_species",
           "read_particle_file", "write_particle_file"]
