"""Discrete adjoint of the device integrator, and a torch.autograd.Function.

The reference has no sensitivities; this is new. A forward run over many
intervals records, per interval, the state at its start (a checkpoint), its
rate constants and every group's accepted step sizes (from the device trace).
With those step sizes held fixed (and, for constrained systems, the line-search
steps of the projection's Newton updates that start each call), each interval
is a smooth map of its start state and the log rate constants through the
projection, the Rosenbrock steps and the clamp;
``adjoint`` walks the intervals backwards, and the device kernel
(``fo_adjoint_interval``) replays each interval from its checkpoint and runs
the reverse stage sweep with transposed solves on the same factorizations and
the mass-action second derivatives.

``Integrate`` wraps the whole thing for torch: Y0 (C, n) and log-rate offsets
theta (R,) in, Y after all intervals out; the rate constants of interval i are
base_i * exp(theta), so dL/dtheta_j sums dL/dlog k_{c,j} over cells and
intervals.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .batch import Batch
from .plan import plan_for
from .solvers import Algorithm


@dataclass
class Trajectory:
    batch: Batch                # the forward state (its plan, groups, options)
    checkpoints: list           # per interval: (n, C) state at its start
    ks: list                    # per interval: (R, C) rate constants
    step_ptr: list              # per interval: (G+1,) int32 device
    steps: list                 # per interval: flat accepted step sizes, device
    max_steps: int
    proj_ptr: list              # per interval: (G+1,) int32 device, or None (no algebraic species)
    proj_steps: list            # per interval: flat line-search steps of the projection's updates
    dt: float
    atol: object                # (n,) device
    statuses: list              # per interval: statuses after the forward call


def forward_record(mech, Y0, k_of, dt, atol, rtol, intervals, group_size=32, algorithm=None, mass=None,
                   trace_cap=512) -> Trajectory:
    """Run the forward integration over `intervals` intervals, recording what
    the adjoint needs. Y0: (C, n) host or device; k_of(i) -> (R, C) device
    tensor (cells fastest) of interval i."""
    import torch
    alg = algorithm if algorithm is not None else Algorithm()
    b = Batch(mech, Y0, group_size=group_size, algorithm=alg, mass=mass, trace_cap=trace_cap)
    at = atol if isinstance(atol, torch.Tensor) else torch.from_numpy(
        np.array(np.broadcast_to(np.asarray(atol, dtype=np.float64), (b.plan.n,)))).to(b.Y.device)
    cps, ks, ptrs, steps, sts, pptrs, psteps = [], [], [], [], [], [], []
    max_steps = 1
    constrained = b.plan.has_constraints
    for i in range(intervals):
        k = k_of(i)
        cps.append(b.Y.clone())
        ks.append(k)
        b.step(k, dt, at, rtol)
        tl = b.trace_len.cpu().numpy()
        if np.any(tl > trace_cap):
            raise RuntimeError(f"interval {i}: more than {trace_cap} attempts in a group; raise trace_cap")
        tr = b.trace.cpu().numpy()
        status = b.statuses()
        ptr, pptr = [0], [0]
        flat, pflat = [], []
        for g in range(b.ngroups):
            rec = tr[g, : tl[g]]
            acc = rec[rec[:, 3] == 1.0, 1]
            flat.extend(acc.tolist())
            ptr.append(len(flat))
            max_steps = max(max_steps, len(acc))
            # the projection's accepted updates; a failed projection restores
            # the state, so none of its updates remain
            if status[g] != "projection failed":
                pflat.extend(rec[rec[:, 3] == 2.0, 1].tolist())
            pptr.append(len(pflat))
        ptrs.append(torch.tensor(ptr, dtype=torch.int32, device=b.Y.device))
        steps.append(torch.tensor(flat if flat else [0.0], dtype=torch.float64, device=b.Y.device))
        if constrained:
            pptrs.append(torch.tensor(pptr, dtype=torch.int32, device=b.Y.device))
            psteps.append(torch.tensor(pflat if pflat else [0.0], dtype=torch.float64, device=b.Y.device))
        else:
            pptrs.append(None)
            psteps.append(None)
        sts.append(status)
    return Trajectory(b, cps, ks, ptrs, steps, max_steps, pptrs, psteps, float(dt), at, sts)


def _workspace(traj: Trajectory):
    import torch
    b = traj.batch
    need = C.c_size_t()
    _abi.check(_abi.lib().fo_adjoint_workspace_bytes(b.plan.handle, b.ngroups, b.max_cells, traj.max_steps,
                                                     C.byref(need)), "fo_adjoint_workspace_bytes")
    return torch.empty(int(need.value), dtype=torch.uint8, device=b.Y.device)


def _call(traj, i, mode, ws, Yin, lam=None, thbar=None, Yout=None, k=None):
    import torch
    b = traj.batch
    Cc = b.C
    st = torch.zeros(b.ngroups, dtype=torch.int32, device=b.Y.device)
    k = traj.ks[i] if k is None else k
    s = torch.cuda.current_stream(b.Y.device)
    rc = _abi.lib().fo_adjoint_interval(
        b.plan.handle, C.byref(b.opts), b.ngroups, b.offsets.data_ptr(), b.max_cells,
        Yin.data_ptr(), 1, Cc, k.data_ptr(), 1, Cc, traj.atol.data_ptr(), traj.dt,
        traj.step_ptr[i].data_ptr(), traj.steps[i].data_ptr(), traj.max_steps,
        traj.proj_ptr[i].data_ptr() if traj.proj_ptr[i] is not None else None,
        traj.proj_steps[i].data_ptr() if traj.proj_steps[i] is not None else None, mode,
        lam.data_ptr() if lam is not None else None, 1, Cc,
        thbar.data_ptr() if thbar is not None else None, 1, Cc,
        Yout.data_ptr() if Yout is not None else None, 1, Cc,
        st.data_ptr(), ws.data_ptr(), ws.numel(), C.c_void_p(s.cuda_stream))
    _abi.check(rc, "fo_adjoint_interval")
    return st


def replay(traj: Trajectory, Y0=None, ks=None):
    """The fixed-step map: integrate from Y0 ((n, C) device; default the
    recorded start) with the recorded step sizes and rate constants `ks`
    (default the recorded ones). Returns the final (n, C) state."""
    import torch
    ws = _workspace(traj)
    Y = (traj.checkpoints[0] if Y0 is None else Y0).clone()
    out = torch.empty_like(Y)
    for i in range(len(traj.checkpoints)):
        st = _call(traj, i, 0, ws, Y, Yout=out, k=None if ks is None else ks[i])
        if np.any(st.cpu().numpy() != 0):
            raise RuntimeError(f"replay of interval {i} failed: {st.cpu().numpy()}")
        Y, out = out, Y
    return Y


def adjoint(traj: Trajectory, lam_final):
    """dL/dY0 ((n, C)) and dL/dlog k per cell ((R, C), summed over intervals)
    from dL/dY at the end ((n, C) device)."""
    import torch
    b = traj.batch
    ws = _workspace(traj)
    lam = lam_final.clone()
    thbar = torch.zeros((b.plan.R, b.C), dtype=torch.float64, device=b.Y.device)
    for i in reversed(range(len(traj.checkpoints))):
        st = _call(traj, i, 1, ws, traj.checkpoints[i], lam=lam, thbar=thbar)
        if np.any(st.cpu().numpy() != 0):
            raise RuntimeError(f"adjoint of interval {i} failed: {st.cpu().numpy()}")
    return lam, thbar


def _torch_function():
    import torch

    class Integrate(torch.autograd.Function):
        """Y_final = integrate(Y0, theta): Y0 (C, n), theta (R,) log-rate
        offsets (k_i = base_i * exp(theta)); spec = dict(mech, base (list of
        (R, C) device tensors, one per interval), dt, atol, rtol, group_size)."""

        @staticmethod
        def forward(ctx, Y0, theta, spec):
            scale = torch.exp(theta.detach())[:, None]
            ks = [kb * scale for kb in spec["base"]]
            traj = forward_record(spec["mech"], Y0.detach(), lambda i: ks[i], spec["dt"], spec["atol"],
                                  spec["rtol"], len(ks), group_size=spec.get("group_size", 32),
                                  algorithm=spec.get("algorithm"))
            ctx.traj = traj
            return traj.batch.Y.t().contiguous()

        @staticmethod
        def backward(ctx, grad_Y):
            lam0, thbar = adjoint(ctx.traj, grad_Y.detach().t().contiguous())
            return lam0.t().contiguous(), thbar.sum(dim=1), None

    return Integrate


_Integrate = None


def integrate(Y0, theta, spec):
    """Differentiable forward integration (see ``Integrate``)."""
    global _Integrate
    if _Integrate is None:
        _Integrate = _torch_function()
    return _Integrate.apply(Y0, theta, spec)
