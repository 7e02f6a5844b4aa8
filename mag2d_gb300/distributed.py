"""Several GPUs, one process each.

Two ways to use them, neither with a collective on the particle data:

* Independent instances (batched sweeps, replicas): instances are split into
  contiguous ranges, one per rank (``shard_range``); every rank advances its
  own with no exchange at all.

* Particle decomposition of one self-consistent instance
  (``ParticleDecomposition``): every rank holds the full grid and a share of
  the particles; after each step the ranks sum the species' fixed-point
  charge deposits (int64, so the sum is bit-identical in any order) with one
  all-reduce, and every rank then solves the same Poisson problem.  With the
  NCCL backend the all-reduce runs in place on the device array that
  mag_rho_fixed_ptr exposes; with gloo it goes through host copies.

Neither the reference (one process, one core) nor this module changes the
physics of a step: a decomposed run equals the single-process run of the
union of the particles, up to the order-free integer deposit.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib


def shard_range(n: int, world: int, rank: int) -> range:
    """Contiguous share of n items for rank of world (sizes differ by at most one)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def allreduce_int64(arr: np.ndarray, group=None) -> np.ndarray:
    """Sum of an int64 array over the ranks of the default (or given) group."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.int64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


class ParticleDecomposition:
    """One self-consistent instance advanced by every rank on its particle share.

    pic: this rank's Pic (the full grid; only this rank's particles loaded).
    """

    def __init__(self, pic, group=None):
        import torch.distributed as dist

        self.pic = pic
        self.group = group
        self.device_reduce = dist.get_backend(group) == "nccl"
        self.nspecies = len(pic.speclist)

    def reduce_deposit(self) -> None:
        """Sum every species' deposit over the ranks and write it back."""
        nx, nz = self.pic.shape
        if self.device_reduce:
            import torch
            import torch.distributed as dist

            self.pic.sync()
            for s in range(self.nspecies):
                ptr = lib().mag_rho_fixed_ptr(self.pic.h, s)
                if not ptr:
                    continue
                t = _device_int64(ptr, nx * nz)
                dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
            torch.cuda.synchronize()
            return
        for s in range(self.nspecies):
            local = self.pic.speclist[s].rho_fixed()
            total = allreduce_int64(local.reshape(-1), self.group).reshape(nx, nz)
            check(lib().mag_set_rho_fixed(self.pic.h, s, total.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))

    def advance_init(self) -> None:
        """Pic::advance_init from the deposit of every rank's particles."""
        self.pic.deposit()
        self.reduce_deposit()
        check(lib().mag_advance_init_ex(self.pic.h, 0))

    def advance(self, n: int = 1) -> None:
        """n steps, each followed by the deposit all-reduce (the next solve sees every rank's charge)."""
        for _ in range(n):
            self.pic.advance(1)
            self.reduce_deposit()


def _device_int64(ptr: int, n: int):
    """A torch view of n int64 in device memory at ptr (no copy)."""
    import torch

    class _Holder:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (int(ptr), False), "version": 3}

    return torch.as_tensor(_Holder(), device="cuda")
