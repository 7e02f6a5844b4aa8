"""torch.autograd binding of the adjoint runs (mag_adjoint_run).

TrapLoss.apply(voltages, bfield, make_pic, nsteps, voltage_keys, checkpoint)
returns the trap diagnostic
    loss = mean axial kinetic energy [eV] + lost fraction
after nsteps steps of a fresh simulation built by make_pic(voltages, bfield)
(a callable returning a Pic with particles loaded and advance_init not yet
called).  Its backward gives d loss / d voltages and d loss / d bfield (the
three components Br, Bt, Bz) from the adjoint of the step computed in the
same forward call, so one forward-backward pass costs one adjoint run instead
of 2 x (parameters) forward runs of finite differences.
"""
from __future__ import annotations

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is present wherever the GPU path runs
    torch = None


if torch is not None:

    class TrapLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, voltages, bfield, make_pic, nsteps, voltage_keys, checkpoint=100):
            v = voltages.detach().cpu().double().numpy()
            b = bfield.detach().cpu().double().numpy()
            pic = make_pic(v, b)
            try:
                info, grad = pic.adjoint(int(nsteps), list(voltage_keys), checkpoint=int(checkpoint), grad_b=True)
            finally:
                pic.close()
            nv = len(voltage_keys)
            ctx.save_for_backward(torch.as_tensor(grad[:nv], dtype=voltages.dtype, device=voltages.device),
                                  torch.as_tensor(grad[nv:nv + 3], dtype=bfield.dtype, device=bfield.device))
            ctx.info = info
            return torch.tensor(info["loss"], dtype=voltages.dtype, device=voltages.device)

        @staticmethod
        def backward(ctx, grad_out):
            gv, gb = ctx.saved_tensors
            return grad_out * gv, grad_out * gb, None, None, None, None

else:  # pragma: no cover
    TrapLoss = None


def loss_from_state(pic, species: int = 0, w_energy: float = 1.0, w_lost: float = 1.0, n0: int | None = None) -> float:
    """The same diagnostic from a plain forward run's final particles (finite differences)."""
    sp = pic.speclist[species]
    g = sp.particles()
    m = sp.info()["mass"]
    e = 0.5 * m * np.asarray(g["vz"], dtype=np.float64) ** 2 / 1.602189e-19
    n_live = len(e)
    lost = 0.0 if not n0 else (n0 - n_live) / n0
    return w_energy * (float(e.mean()) if n_live else 0.0) + w_lost * lost
