"""Batched, device-resident integration of many groups of one mechanism.

``Batch`` keeps the state of C cells on the GPU in the species-major layout
(n, C), cells fastest, with one controller memory, one counter row and one
status per group, and integrates every group over an interval with a single
``fo_solve`` launch. It is the device-side form of the reference's scenario
loop (fastode/ts1.py:196-222): per group a Memory carried across intervals,
per interval fresh rate constants.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .counts import COUNT_FIELDS, Counts
from .plan import plan_for
from .solvers import Algorithm


def group_offsets(n_cells: int, group_size: int) -> np.ndarray:
    """Contiguous groups of `group_size` cells; the last one may be short
    (fastode/ts1.py:196-197)."""
    starts = list(range(0, n_cells, group_size)) + [n_cells]
    return np.array(starts, dtype=np.int32)


class Batch:
    def __init__(self, mech, Y0, group_size: int = 32, algorithm: Algorithm = None, mass=None,
                 offsets=None, slots: int = 0, trace_cap: int = 0, stream=None):
        import torch
        self.torch = torch
        self.alg = algorithm if algorithm is not None else Algorithm()
        self.plan = plan_for(mech, mass, self.alg.ordering, getattr(self.alg, "tile", 6))
        dev = torch.device("cuda", self.plan.device)
        self.dev = dev
        Y0 = Y0 if isinstance(Y0, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(Y0, dtype=np.float64))
        self.C, n = Y0.shape
        if n != self.plan.n:
            raise ValueError(f"Y0 has {n} species, the mechanism {self.plan.n}")
        offs = group_offsets(self.C, group_size) if offsets is None else np.asarray(offsets, dtype=np.int32)
        self.offsets_host = offs
        self.ngroups = len(offs) - 1
        self.max_cells = int(np.max(np.diff(offs)))
        self.offsets = torch.from_numpy(offs).to(dev)
        self.Y = Y0.to(dev, dtype=torch.float64).t().contiguous()          # (n, C)
        self.memory = torch.zeros((self.ngroups, 3), dtype=torch.float64, device=dev)
        self.counts = torch.zeros((self.ngroups, len(COUNT_FIELDS)), dtype=torch.int64, device=dev)
        self.status = torch.zeros(self.ngroups, dtype=torch.int32, device=dev)
        self.slots = int(slots)
        grid = self.ngroups if self.slots <= 0 else min(self.slots, self.ngroups)
        self.ws = torch.empty(self.plan.workspace_bytes(grid, self.max_cells), dtype=torch.uint8, device=dev)
        self.trace_cap = int(trace_cap)
        if self.trace_cap > 0:
            self.trace = torch.zeros((self.ngroups, self.trace_cap, 4), dtype=torch.float64, device=dev)
            self.trace_len = torch.zeros(self.ngroups, dtype=torch.int32, device=dev)
        self.opts = self.plan.options_for(self.alg, self.max_cells)
        self.stream = stream

    def _stream(self):
        s = self.stream if self.stream is not None else self.torch.cuda.current_stream(self.dev)
        return s

    def step(self, k, dt: float, atol, rtol: float) -> None:
        """Integrate every group over one interval of length dt, asynchronously
        on the batch's stream. k: device tensor (R, C), cells fastest; atol:
        device tensor (n,)."""
        s = self._stream()
        rc = _abi.lib().fo_solve(
            self.plan.handle, C.byref(self.opts), self.ngroups, self.offsets.data_ptr(), self.max_cells,
            self.Y.data_ptr(), 1, self.C, k.data_ptr(), 1, self.C,
            atol.data_ptr(), float(rtol), float(dt),
            self.memory.data_ptr(), self.counts.data_ptr(), self.status.data_ptr(),
            self.ws.data_ptr(), self.ws.numel(), self.slots,
            self.trace.data_ptr() if self.trace_cap else None, self.trace_cap,
            self.trace_len.data_ptr() if self.trace_cap else None, C.c_void_p(s.cuda_stream))
        _abi.check(rc, "fo_solve")

    def state(self) -> np.ndarray:
        """The cells' state as (C, n) on the host."""
        return self.Y.t().contiguous().cpu().numpy()

    def total_counts(self) -> Counts:
        c = Counts()
        for row in self.counts.cpu().numpy():
            c.add_row(row)
        return c

    def statuses(self) -> list:
        return [_abi.STATUS_STRINGS[int(s)] for s in self.status.cpu().numpy()]


class HostState:
    """Device buffers and per-group controller memory carried between
    ``solve_host`` calls (the reference's per-group Memory of
    fastode/ts1.py:201, kept on the device)."""

    def __init__(self, mech, C_cells, n, R, group_size, algorithm, mass, slots, dev):
        import torch
        self.alg = algorithm if algorithm is not None else Algorithm()
        self.plan = plan_for(mech, mass, self.alg.ordering, getattr(self.alg, "tile", 6))
        offs = group_offsets(C_cells, group_size)
        self.ngroups = len(offs) - 1
        self.max_cells = int(np.max(np.diff(offs)))
        self.offsets = torch.from_numpy(offs).to(dev)
        self.Y = torch.empty((C_cells, n), dtype=torch.float64, device=dev)
        self.k = torch.empty((C_cells, R), dtype=torch.float64, device=dev)
        self.atol = torch.empty(n, dtype=torch.float64, device=dev)
        self.memory = torch.zeros((self.ngroups, 3), dtype=torch.float64, device=dev)
        self.counts = torch.zeros((self.ngroups, len(COUNT_FIELDS)), dtype=torch.int64, device=dev)
        self.status = torch.zeros(self.ngroups, dtype=torch.int32, device=dev)
        self.slots = int(slots)
        grid = self.ngroups if self.slots <= 0 else min(self.slots, self.ngroups)
        self.ws = torch.empty(self.plan.workspace_bytes(grid, self.max_cells), dtype=torch.uint8, device=dev)
        self.Y_out = torch.empty((C_cells, n), dtype=torch.float64).pin_memory()
        self.status_out = torch.empty(self.ngroups, dtype=torch.int32).pin_memory()
        self.opts = self.plan.options_for(self.alg, self.max_cells)
        self.shape = (C_cells, n, R)
        self._overlap = None

    def overlap_buffers(self):
        """The second stream and the extra buffers of ``solve_host_intervals``
        (a second rate-constant buffer, two staging states, a second pinned
        output), made on first use and kept."""
        import torch
        if self._overlap is None:
            dev = self.Y.device
            self._overlap = {
                "side": torch.cuda.Stream(dev),
                "kbuf": [self.k, torch.empty_like(self.k)],
                "stage": [torch.empty_like(self.Y) for _ in range(2)],
                "stage_st": [torch.empty_like(self.status) for _ in range(2)],
                "yout": [self.Y_out, torch.empty(self.Y_out.shape, dtype=torch.float64).pin_memory()],
                "stout": [self.status_out, torch.empty(self.status_out.shape, dtype=torch.int32).pin_memory()],
            }
        return self._overlap


def solve_host(mech, Y, k, dt, atol, rtol, state: HostState = None, group_size: int = 32,
               algorithm: Algorithm = None, mass=None, slots: int = 0):
    """Integrate the cells of host arrays Y (C, n) and k (C, R), both in the
    reference's cell-major layout, over one interval, in groups of
    `group_size` cells that each carry their own controller memory from call
    to call in `state`. Returns (Y_new (C, n) host tensor, state,
    (bytes host-to-device, bytes device-to-host)). Pinned host tensors copy
    fastest. The statuses of the call are in ``state.status_out``."""
    import torch
    Yt = Y if isinstance(Y, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(Y, dtype=np.float64))
    kt = k if isinstance(k, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(k, dtype=np.float64))
    C_cells, n = Yt.shape
    R = kt.shape[1]
    if state is None:
        dev = torch.device("cuda", torch.cuda.current_device())
        state = HostState(mech, C_cells, n, R, group_size, algorithm, mass, slots, dev)
    if state.shape != (C_cells, n, R):
        raise ValueError("state was made for other shapes")
    s = torch.cuda.current_stream(state.Y.device)
    state.Y.copy_(Yt, non_blocking=True)
    state.k.copy_(kt, non_blocking=True)
    at = torch.from_numpy(np.array(np.broadcast_to(np.asarray(atol, dtype=np.float64), (n,))))
    state.atol.copy_(at, non_blocking=False)
    rc = _abi.lib().fo_solve(
        state.plan.handle, C.byref(state.opts), state.ngroups, state.offsets.data_ptr(), state.max_cells,
        state.Y.data_ptr(), n, 1, state.k.data_ptr(), R, 1, state.atol.data_ptr(), float(rtol), float(dt),
        state.memory.data_ptr(), state.counts.data_ptr(), state.status.data_ptr(),
        state.ws.data_ptr(), state.ws.numel(), state.slots, None, 0, None, C.c_void_p(s.cuda_stream))
    _abi.check(rc, "fo_solve")
    state.Y_out.copy_(state.Y, non_blocking=True)
    state.status_out.copy_(state.status, non_blocking=True)
    s.synchronize()
    h2d = Yt.numel() * 8 + kt.numel() * 8 + n * 8
    d2h = state.Y_out.numel() * 8 + state.status_out.numel() * 4
    return state.Y_out, state, (h2d, d2h)


def solve_host_intervals(mech, Y, ks, dt, atol, rtol, state: HostState = None, group_size: int = 32,
                         algorithm: Algorithm = None, mass=None, slots: int = 0, on_result=None):
    """``solve_host`` over several intervals with the copies overlapped: Y
    (C, n) is the host state at the start and ks a sequence of host (C, R)
    rate-constant arrays, one per interval. The state stays on the device
    between intervals; each interval's rate constants are copied in on a
    second stream while the previous interval integrates, and each
    interval's state and statuses are copied out on that stream while the
    next one integrates. on_result(i, Y_host, status_host), when given, is
    called with every interval's result as soon as it is on the host; both
    tensors are pinned buffers that are overwritten two intervals later (copy
    them to keep them). Returns (the last interval's Y as a host tensor,
    state, (bytes host-to-device, bytes device-to-host))."""
    import torch
    ks = list(ks)
    if not ks:
        raise ValueError("no intervals")

    def host(a):
        return a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64))

    Yt = host(Y)
    C_cells, n = Yt.shape
    R = host(ks[0]).shape[1]
    if state is None:
        dev = torch.device("cuda", torch.cuda.current_device())
        state = HostState(mech, C_cells, n, R, group_size, algorithm, mass, slots, dev)
    if state.shape != (C_cells, n, R):
        raise ValueError("state was made for other shapes")
    dev = state.Y.device
    comp = torch.cuda.current_stream(dev)
    ob = state.overlap_buffers()
    side, kbuf, stage, stage_st, yout, stout = (ob[k] for k in ("side", "kbuf", "stage", "stage_st", "yout", "stout"))
    side.wait_stream(comp)                        # the buffers' last users were on the compute stream
    at = torch.from_numpy(np.array(np.broadcast_to(np.asarray(atol, dtype=np.float64), (n,))))
    state.atol.copy_(at, non_blocking=False)
    state.Y.copy_(Yt, non_blocking=True)
    kbuf[0].copy_(host(ks[0]), non_blocking=True)
    k_ready = [None, None]
    solved = [None] * len(ks)
    copied = [None] * len(ks)
    h2d = Yt.numel() * 8 + n * 8 + host(ks[0]).numel() * 8
    d2h = 0

    def deliver(j):
        copied[j].synchronize()
        if on_result is not None:
            on_result(j, yout[j % 2], stout[j % 2])

    for i in range(len(ks)):
        if i + 1 < len(ks):                       # rate constants of the next interval
            kn = host(ks[i + 1])
            with torch.cuda.stream(side):
                if i >= 1:
                    side.wait_event(solved[i - 1])   # its buffer was interval i-1's
                kbuf[(i + 1) % 2].copy_(kn, non_blocking=True)
                k_ready[(i + 1) % 2] = side.record_event()
            h2d += kn.numel() * 8
        if i >= 1:
            comp.wait_event(k_ready[i % 2])
        kb = kbuf[i % 2]
        rc = _abi.lib().fo_solve(
            state.plan.handle, C.byref(state.opts), state.ngroups, state.offsets.data_ptr(), state.max_cells,
            state.Y.data_ptr(), n, 1, kb.data_ptr(), R, 1, state.atol.data_ptr(), float(rtol), float(dt),
            state.memory.data_ptr(), state.counts.data_ptr(), state.status.data_ptr(),
            state.ws.data_ptr(), state.ws.numel(), state.slots, None, 0, None, C.c_void_p(comp.cuda_stream))
        _abi.check(rc, "fo_solve")
        if i >= 2:
            comp.wait_event(copied[i - 2])        # the staging buffers' previous copy-out
        stage[i % 2].copy_(state.Y)
        stage_st[i % 2].copy_(state.status)
        solved[i] = comp.record_event()
        with torch.cuda.stream(side):
            side.wait_event(solved[i])
            yout[i % 2].copy_(stage[i % 2], non_blocking=True)
            stout[i % 2].copy_(stage_st[i % 2], non_blocking=True)
            copied[i] = side.record_event()
        d2h += yout[i % 2].numel() * 8 + stout[i % 2].numel() * 4
        if i >= 1:
            deliver(i - 1)
    deliver(len(ks) - 1)
    comp.wait_stream(side)
    return yout[(len(ks) - 1) % 2], state, (h2d, d2h)
