"""The drop-in integrator: ``Algorithm(ROS3|RODAS3).solve(system, Y, dt, atol,
rtol, counts, memory)`` with the reference's signature, options, ``Memory``,
``Counts`` accumulation and status strings (fastode/solvers.py:181-186,
270-415), running on the GPU through the C-ABI.

What stays on the host is bookkeeping only: copying the group's state and rate
constants to the device, one ``fo_solve`` call, and copying the clamped state,
the controller memory, the counters and the status back. The stage loop, the
error norm, the controller, the LU and the mechanism evaluations all run in
the library's kernels; a system the kernels cannot run (anything but a
mass-action ``ChemSystem``) is rejected with ``TypeError`` instead of being
integrated on the CPU.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from .counts import Counts
from .plan import plan_for
from .tableaus import ROS3, RODAS3, Tableau

H_MIN_FRACTION = 1.0e-15
H_START_FRACTION = 1.0e-6
ERROR_MIN = 1.0e-10


@dataclass
class Memory:
    """What the integrator carries from one interval to the next
    (fastode/solvers.py:181-186)."""
    h_next: float = 0.0
    err_prev: float = 0.0
    h_prev: float = 0.0


def quantize(h: float, interval: float) -> float:
    """Round h down to a divisor of the interval (fastode/solvers.py:46-51);
    the device applies the same rule to every proposal."""
    if h >= interval:
        return interval
    n = math.ceil(interval / h - 1.0e-9)
    return interval / max(n, 1)


def tableau_id(tab) -> int:
    name = getattr(tab, "name", str(tab)).lower()
    if name == "ros3":
        return 0
    if name == "rodas3":
        return 1
    raise ValueError(f"unknown tableau {name!r}: the device integrator has ROS3 and RODAS3")


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("fastode_gb300 needs a CUDA GPU: there is no host integrator")
    return torch


def _require_chem(system):
    if getattr(system, "mech", None) is None or getattr(system, "k", None) is None:
        raise TypeError("the GPU integrator runs mass-action ChemSystem objects only "
                        f"(got {type(system).__name__}); there is no CPU fallback")


def _k_rows(system, C_cells: int) -> np.ndarray:
    k = np.atleast_2d(np.asarray(system.k, dtype=np.float64))
    if k.shape[0] not in (1, C_cells):
        raise ValueError(f"k has {k.shape[0]} rows for {C_cells} cells")
    return np.ascontiguousarray(k)


def _device_solve(solver, system, Y, dt, atol, rtol, counts: Counts, mem):
    """One fo_solve call on one group: the host side of every solver's
    ``solve``. ``mem`` is a Memory updated in place, or None when the loop
    carries nothing (its device copy is then neither read nor written)."""
    _require_chem(system)
    torch = _torch()
    Y = np.asarray(Y, dtype=np.float64)
    if Y.ndim != 2:
        raise ValueError("Y must have shape (cells, species)")
    C_cells, n = Y.shape
    if n != system.n:
        raise ValueError(f"Y has {n} species, the system {system.n}")
    plan = plan_for(system.mech, system.mass, solver.ordering, getattr(solver, "tile", 6))
    k = _k_rows(system, C_cells)
    atol = np.array(np.broadcast_to(np.asarray(atol, dtype=np.float64), (n,)))
    dev = torch.device("cuda", plan.device)
    Yd = torch.from_numpy(np.ascontiguousarray(Y)).to(dev)
    kd = torch.from_numpy(k).to(dev)
    atold = torch.from_numpy(atol).to(dev)
    m = mem if mem is not None else Memory()
    memd = torch.tensor([m.h_next, m.err_prev, m.h_prev], dtype=torch.float64, device=dev)
    cnt = torch.zeros((1, _abi.NUM_COUNTS), dtype=torch.int64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    offs = torch.tensor([0, C_cells], dtype=torch.int32, device=dev)
    ws = plan.workspace(1, C_cells)
    stream = torch.cuda.current_stream(dev)
    rc = _abi.lib().fo_solve(
        plan.handle, C.byref(plan.options_for(solver, C_cells)), 1, offs.data_ptr(), C_cells,
        Yd.data_ptr(), n, 1, kd.data_ptr(), 0 if k.shape[0] == 1 else plan.R, 1,
        atold.data_ptr(), float(rtol), float(dt),
        memd.data_ptr(), cnt.data_ptr(), st.data_ptr(), ws.data_ptr(), ws.numel(), 0,
        None, 0, None, C.c_void_p(stream.cuda_stream))
    _abi.check(rc, "fo_solve")
    stream.synchronize()
    if mem is not None:
        h = memd.cpu().numpy()
        mem.h_next, mem.err_prev, mem.h_prev = float(h[0]), float(h[1]), float(h[2])
    counts.add_row(cnt.cpu().numpy()[0])
    return Yd.cpu().numpy(), _abi.STATUS_STRINGS[int(st.cpu().item())]


class Algorithm:
    """The integrator of the reference's Section 4 (fastode/solvers.py:270-415)."""

    name = "algorithm"

    def __init__(self, tableau: Tableau = ROS3, controller: str = "h211b", b: float = 4.0,
                 safety: float = 0.9, fac_min: float = 0.2, fac_max: float = 6.0,
                 carry: bool = True, quantize: bool = True, max_steps: int = 1000,
                 carry_memory: bool = True, ordering: str = "auto", kernel: str = "generated", tile: int = 6,
                 lockstep: bool = True):
        """The reference's arguments, plus those of the device path: the
        fill-reducing ``ordering`` of the sparse LU and the ``kernel`` variant:
        "generated", the mechanism's own factorization and solves generated as
        straight-line code when its plan is first used (compiled once, then
        cached on disk; groups of at most 32 cells, larger groups run
        "compact"); "compact", table-driven, half a row and half the solve
        vector in shared memory; "pipelined", whole rows in shared memory; or
        "plain", the direct loops. All give the same factors; "generated" and
        "plain" give the same solutions bit for bit, the others differ in the
        solves' summation order. ``tile``: the generated factorization's
        register tiles (rows and columns), a speed choice only. ``lockstep``:
        with the generated kernel and one block per group, the groups make
        their attempts in rounds in a cooperative launch (fo_options.lockstep),
        also a speed choice only."""
        self.tableau = tableau
        self.controller = controller
        self.b = b
        self.safety = safety
        self.fac_min = fac_min
        self.fac_max = fac_max
        self.carry = carry
        self.quantize = quantize
        self.max_steps = max_steps
        self.carry_memory = carry_memory
        self.ordering = ordering
        if kernel not in _abi.VARIANTS:
            raise ValueError(f"kernel must be one of {sorted(_abi.VARIANTS)}")
        self.kernel = kernel
        self.tile = int(tile)
        self.lockstep = bool(lockstep)
        tableau_id(tableau)

    def new_memory(self) -> Memory:
        return Memory()

    def factor(self, err: float, H: float, mem: Memory) -> float:
        """The step factor after an accepted step (fastode/solvers.py:297-303);
        the device evaluates the same expression."""
        k = float(self.tableau.k)
        fac = self.safety / err ** (1.0 / k)
        if self.controller == "h211b" and mem.err_prev > 0.0 and mem.h_prev > 0.0:
            fac = (self.safety * (err * mem.err_prev) ** (-1.0 / (self.b * k))
                   * (H / mem.h_prev) ** (-1.0 / self.b))
        return min(self.fac_max, max(self.fac_min, fac))

    def options(self) -> _abi.Options:
        return _abi.Options(tableau_id(self.tableau), 0 if self.controller == "h211b" else 1,
                            float(self.b), float(self.safety), float(self.fac_min), float(self.fac_max),
                            int(bool(self.carry)), int(bool(self.quantize)), int(bool(self.carry_memory)),
                            int(self.max_steps), _abi.VARIANTS[self.kernel], 0, 0,
                            lockstep=int(getattr(self, "lockstep", False)))

    def solve(self, system, Y, dt, atol, rtol, counts: Counts, memory: Memory = None):
        """Integrate one group (all rows of Y) over one interval; returns
        (Y_new, status). Y is copied, ``counts`` accumulated and ``memory``
        updated in place, as in the reference."""
        return _device_solve(self, system, Y, dt, atol, rtol, counts,
                             memory if memory is not None else Memory())


class RestartingLoop(Algorithm):
    """The baseline Rosenbrock loop of fastode/solvers.py:189-267 on the GPU:
    restarted at 1e-6 of the interval every call under the elementary
    controller, no memory carried (``new_memory`` returns None, as in the
    reference). step_change_rows: with constraints, the step change replaces
    the algebraic rows of the error estimate."""

    name = "restarting"

    def __init__(self, tableau: Tableau = ROS3, max_steps: int = 1000, step_change_rows: bool = True,
                 ordering: str = "auto", kernel: str = "generated", tile: int = 6):
        super().__init__(tableau, controller="elementary", max_steps=max_steps, ordering=ordering, kernel=kernel,
                         tile=tile)
        self.step_change_rows = step_change_rows

    def new_memory(self):
        return None

    def options(self) -> _abi.Options:
        o = super().options()
        o.loop = 1
        o.step_change_rows = int(bool(self.step_change_rows))
        return o

    def solve(self, system, Y, dt, atol, rtol, counts: Counts, memory=None):
        """Integrate one group over one interval; returns (Y_new, status)."""
        return _device_solve(self, system, Y, dt, atol, rtol, counts, None)


class BackwardEuler:
    """The baseline backward Euler with a full Newton iteration
    (fastode/solvers.py:418-491) on the GPU: every Newton iteration evaluates
    the rhs and Jacobian, factors M/H - J and solves once; a failed step is
    retried from the last accepted state with H cut by the next reduction,
    and past the last reduction the unconverged iterate is accepted
    ("accepted unconverged"). Counts newton, failures and unconverged as the
    reference does. ``max_steps`` is a guard the reference does not have (its
    loop has no budget): a group that takes more steps in one call reports
    "too many steps". ``ordering`` and ``kernel`` choose the device LU as for
    Algorithm."""

    name = "backward-euler"

    def __init__(self, max_iterations: int = 11, reductions=(0.5, 0.5, 0.5, 0.5, 0.1),
                 small: float = 1.0e-40, max_steps: int = 1_000_000, ordering: str = "auto",
                 kernel: str = "generated", tile: int = 6):
        self.max_iterations = max_iterations
        self.reductions = tuple(float(r) for r in reductions)
        if len(self.reductions) > 8:
            raise ValueError("the device loop takes at most 8 reductions")
        if not all(r > 0.0 and math.isfinite(r) for r in self.reductions):
            raise ValueError("reductions must be positive and finite")
        self.small = small
        self.max_steps = max_steps
        self.ordering = ordering
        if kernel not in _abi.VARIANTS:
            raise ValueError(f"kernel must be one of {sorted(_abi.VARIANTS)}")
        self.kernel = kernel
        self.tile = int(tile)

    def new_memory(self):
        return None

    def converged(self, delta, Y, atol, rtol) -> bool:
        """The Newton convergence test (fastode/solvers.py:432-437), as the
        device applies it to every iterate of a group."""
        if not np.all(np.isfinite(delta)):
            return False
        bound = np.maximum(np.maximum(self.small, np.asarray(atol)[None, :]), rtol * np.abs(Y))
        return bool(np.all(np.abs(delta) <= bound))

    def options(self) -> _abi.Options:
        o = _abi.Options()
        o.tableau = 0
        o.controller = 1
        o.max_steps = int(self.max_steps)
        o.variant = _abi.VARIANTS[self.kernel]
        o.loop = _abi.LOOPS["backward-euler"]
        o.max_iterations = int(self.max_iterations)
        o.nreductions = len(self.reductions)
        for i, r in enumerate(self.reductions):
            o.reductions[i] = r
        o.small = float(self.small)
        return o

    def solve(self, system, Y, dt, atol, rtol, counts: Counts, memory=None):
        """Integrate one group over one interval; returns (Y_new, status)."""
        return _device_solve(self, system, Y, dt, atol, rtol, counts, None)


def _eval(system, Y, jac: bool):
    _require_chem(system)
    torch = _torch()
    Y = np.ascontiguousarray(np.asarray(Y, dtype=np.float64))
    C_cells, n = Y.shape
    plan = plan_for(system.mech, system.mass)
    k = _k_rows(system, C_cells)
    dev = torch.device("cuda", plan.device)
    Yd = torch.from_numpy(Y).to(dev)
    kd = torch.from_numpy(k).to(dev)
    out = torch.empty((C_cells, plan.nnz if jac else n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    f = _abi.lib().fo_eval_jac if jac else _abi.lib().fo_eval_rhs
    rc = f(plan.handle, C_cells, Yd.data_ptr(), n, 1, kd.data_ptr(), 0 if k.shape[0] == 1 else plan.R, 1,
           out.data_ptr(), C.c_void_p(stream.cuda_stream))
    _abi.check(rc, "fo_eval_jac" if jac else "fo_eval_rhs")
    return out.cpu().numpy()


def device_rhs(system, Y):
    """F(Y) on the GPU (fastode/chem.py:89-90)."""
    return _eval(system, Y, jac=False)


def device_jac(system, Y):
    """Jacobian values on the pattern on the GPU (fastode/chem.py:92-102)."""
    return _eval(system, Y, jac=True)
