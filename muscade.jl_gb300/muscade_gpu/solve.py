"""`solve(SweepXGPU{OX}; ...)`: the drop-in solver over the device path.

Mirrors the reference's solver entry (src/Solve.jl:16-35) and SweepX keywords
(src/SweepX.jl:179-184): `time`, `initialstate`, `β`, `γ`, `maxiter`, `maxΔx`,
`maxLλ`.  Returns the list of states, one per time step.  On failure the
states of the converged steps are kept in `pstate` (like the reference's
partial results) and a `MuscadeError` carries the reference's message.
"""
from __future__ import annotations

import math

import numpy as np

from .device import DeviceError, DeviceModel
from .model import MuscadeError, State


class SweepXGPU:
    """Solver type SweepXGPU{OX}; use SweepXGPU[0] or SweepXGPU[2]."""

    def __class_getitem__(cls, OX):
        if OX not in (0, 2):
            raise MuscadeError("SweepXGPU supports OX=0 (static) and OX=2 (Newmark-β)")
        return type(f"SweepXGPU{{{OX}}}", (cls,), {"OX": OX})


def solve(solver, initialstate: State, time, beta=0.25, gamma=0.5, maxiter=50, maxdx=1e-5, maxLl=math.inf,
          pstate=None, device: int = 0, devmodel: DeviceModel | None = None, verbose=False, linsolve="auto"):
    """`linsolve` picks the device linear solver: 'auto', 'f32ir', 'f64', 'block',
    'torn', 'torn32', 'sparse' or 'sparse64' (see DeviceModel.set_linear_solver);
    it is ignored when `devmodel` is given."""
    OX = solver.OX
    model, dis = initialstate.model, initialstate.dis
    dm = devmodel or DeviceModel(model, dis, device=device, linsolve=linsolve)
    try:
        if dm.nA:
            dm.set_A(initialstate.A)
        X0 = list(initialstate.X)[: OX + 1]
        rc, states, stats = dm.sweepx(OX, np.asarray(time, dtype=np.float64), initialstate.time, X0,
                                      U=initialstate.U[0], beta=beta, gamma=gamma, maxiter=maxiter, maxdx=maxdx,
                                      maxLl=maxLl)
        out = []
        for k in range(stats.nstep_done):
            s = initialstate.copy(nXder=OX + 1)
            s.time = float(time[k])
            s.X = tuple(states[k, d].copy() for d in range(OX + 1))
            out.append(s)
        if pstate is not None:
            pstate[:] = out
        if rc != 0:
            raise DeviceError(rc, dm.lib.mgpu_last_error(dm.ctx).decode(errors="replace"))
        if verbose:
            print(f"    nel={model.nele()}, ndof={model.ndof['X']}, nstep={len(time)}, niter={stats.niter_total}, "
                  f"niter/nstep={stats.niter_total / max(len(time), 1):5.2f}")
        return out
    finally:
        if devmodel is None:
            dm.close()
