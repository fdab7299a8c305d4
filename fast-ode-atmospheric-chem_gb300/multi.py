"""Several mechanisms in one persistent launch per interval, replayed as a CUDA graph.

A ``Part`` is one mechanism's cells: state (n, C) and rate constants (R, C) in
HBM with cells fastest, per-group controller memory, counters and statuses, and
optionally the photolysis columns that follow the diurnal factor. ``MultiBatch``
integrates every part over an interval with one ``fo_multi_launch`` (blocks pull
groups of all mechanisms from one device queue, largest mechanism first; with
the generated kernel, one module holds every mechanism's own factorization and
solves) after
one photolysis update per part; the interval's time lives on the device, so the
same captured CUDA graph replays every interval. This is the device form of the
reference's scenario loop (fastode/ts1.py:196-222) over several mechanisms.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from .batch import group_offsets
from .counts import COUNT_FIELDS, Counts
from .plan import plan_for
from .solvers import Algorithm

SMEM_PER_SM = 232448


class Part:
    def __init__(self, mech, Y0, k, atol, rtol, dt, group_size=32, algorithm=None, mass=None,
                 photolysis=None, device=None):
        """Y0 (C, n) and k (C, R) host arrays (or device tensors) in the
        reference's layout; photolysis = (reaction indices, J, per-cell phase)
        for the reactions whose k follows J * max(0, cos(phase + omega t))."""
        import torch
        self.alg = algorithm if algorithm is not None else Algorithm()
        self.plan = plan_for(mech, mass, self.alg.ordering, getattr(self.alg, "tile", 6))
        dev = device if device is not None else torch.device("cuda", self.plan.device)
        Y0 = torch.as_tensor(np.asarray(Y0, dtype=np.float64)) if not isinstance(Y0, torch.Tensor) else Y0
        k = torch.as_tensor(np.asarray(k, dtype=np.float64)) if not isinstance(k, torch.Tensor) else k
        self.C, self.n = Y0.shape
        self.R = k.shape[1]
        self.Y0 = Y0.to(dev).t().contiguous()
        self.Y = self.Y0.clone()
        self.k = k.to(dev).t().contiguous()
        self.atol = torch.as_tensor(np.broadcast_to(np.asarray(atol, dtype=np.float64), (self.n,)).copy()).to(dev)
        self.rtol, self.dt = float(rtol), float(dt)
        offs = group_offsets(self.C, group_size)
        self.group_size = int(group_size)
        self.ngroups = len(offs) - 1
        self.max_cells = int(np.max(np.diff(offs)))
        self.offsets = torch.from_numpy(offs).to(dev)
        self.memory = torch.zeros((self.ngroups, 3), dtype=torch.float64, device=dev)
        self.counts = torch.zeros((self.ngroups, len(COUNT_FIELDS)), dtype=torch.int64, device=dev)
        self.status = torch.zeros(self.ngroups, dtype=torch.int32, device=dev)
        self.photo = None
        if photolysis is not None:
            rxn, J, phase = photolysis
            self.photo = (torch.as_tensor(np.asarray(rxn, dtype=np.int32)).to(dev),
                          torch.as_tensor(np.asarray(J, dtype=np.float64)).to(dev),
                          torch.as_tensor(np.asarray(phase, dtype=np.float64)).to(dev))

    def desc(self) -> _abi.BatchDesc:
        o = self.alg.options()
        if o.variant == _abi.VARIANTS["generated"] and self.max_cells > 32:
            o.variant = _abi.VARIANTS["compact"]     # generated code runs groups of at most 32 cells
        return _abi.BatchDesc(self.plan.handle.value, o, self.ngroups, self.offsets.data_ptr(),
                              self.max_cells, self.Y.data_ptr(), 1, self.C, self.k.data_ptr(), 1, self.C,
                              self.atol.data_ptr(), self.rtol, self.dt, self.memory.data_ptr(),
                              self.counts.data_ptr(), self.status.data_ptr())

    def smem_per_block(self) -> int:
        lanes = ((self.max_cells + 31) // 32) * 32
        kernel = getattr(self.alg, "kernel", "pipelined")
        if kernel == "generated" and self.max_cells <= 32:
            # the reduction buffer, and the projection's work row of a constrained mechanism
            return 8 * (32 + (self.n * lanes if self.plan.has_constraints else 0))
        return 8 * (32 + self.plan.smem_items("compact" if kernel == "generated" else kernel) * lanes)

    def generated(self) -> bool:
        return getattr(self.alg, "kernel", "") == "generated" and self.max_cells <= 32

    def reset(self):
        self.Y.copy_(self.Y0)
        self.memory.zero_()
        self.counts.zero_()
        self.status.zero_()

    def state(self) -> np.ndarray:
        return self.Y.t().contiguous().cpu().numpy()

    def total_counts(self) -> Counts:
        c = Counts()
        for row in self.counts.cpu().numpy():
            c.add_row(row)
        return c


def default_slots(parts, device_index: int) -> int:
    """Persistent blocks: as many as shared memory lets each SM hold, times the
    SM count."""
    import torch
    sms = torch.cuda.get_device_properties(device_index).multi_processor_count
    smem = max(p.smem_per_block() for p in parts)
    # the generated kernel is register-bound at sixteen one-warp blocks per
    # SM (128 registers per thread); the table-driven ones at eight
    cap = 16 if all(p.generated() for p in parts) else 8
    per_sm = max(1, min(cap, SMEM_PER_SM // smem))
    return sms * per_sm


class MultiBatch:
    OMEGA = 2.0 * math.pi / 86400.0

    def __init__(self, parts, slots: int = 0, t0: float = 0.0):
        import torch
        self.torch = torch
        self.parts = list(parts)
        dev = self.parts[0].Y.device
        self.dev = dev
        self.slots = int(slots) if slots else default_slots(self.parts, dev.index)
        descs = (_abi.BatchDesc * len(self.parts))(*[p.desc() for p in self.parts])
        self._descs = descs
        need = C.c_size_t()
        _abi.check(_abi.lib().fo_multi_workspace_bytes(len(self.parts), descs, self.slots, C.byref(need)),
                   "fo_multi_workspace_bytes")
        self.ws = torch.empty(int(need.value), dtype=torch.uint8, device=dev)
        handle = C.c_void_p()
        _abi.check(_abi.lib().fo_multi_prepare(len(self.parts), descs, self.ws.data_ptr(), self.ws.numel(),
                                               self.slots, C.byref(handle)), "fo_multi_prepare")
        self.handle = handle
        self.t = torch.full((1,), float(t0), dtype=torch.float64, device=dev)
        self.dt = self.parts[0].dt
        if any(p.dt != self.dt for p in self.parts):
            raise ValueError("all parts of a MultiBatch share the interval length")
        self.graph = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            _abi.lib().fo_multi_destroy(h)

    def enqueue_interval(self, stream=None):
        """Photolysis for every part at the device clock, one persistent
        integrator launch, clock += dt; all asynchronous on `stream`."""
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev)
        sp = C.c_void_p(s.cuda_stream)
        lib = _abi.lib()
        for p in self.parts:
            if p.photo is not None:
                rxn, J, phase = p.photo
                _abi.check(lib.fo_update_photolysis_clock(p.C, rxn.numel(), rxn.data_ptr(), J.data_ptr(),
                                                          phase.data_ptr(), self.OMEGA, self.t.data_ptr(),
                                                          p.k.data_ptr(), 1, p.C, sp), "fo_update_photolysis_clock")
        _abi.check(lib.fo_multi_launch(self.handle, sp), "fo_multi_launch")
        _abi.check(lib.fo_advance_clock(self.t.data_ptr(), self.dt, sp), "fo_advance_clock")

    def launches_per_interval(self) -> int:
        return sum(1 for p in self.parts if p.photo is not None) + 2

    def capture(self):
        """Capture one interval as a CUDA graph (on a side stream, as CUDA
        graph capture requires)."""
        torch = self.torch
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.dev)
        s.wait_stream(torch.cuda.current_stream(self.dev))
        torch.cuda.synchronize(self.dev)
        t_saved = self.t.clone()
        states = [(p.Y.clone(), p.memory.clone(), p.counts.clone(), p.status.clone(), p.k.clone())
                  for p in self.parts]
        with torch.cuda.stream(s):
            self.enqueue_interval(s)          # warm-up outside the graph: sets kernel attributes
        torch.cuda.synchronize(self.dev)
        for p, (Y, m, c, st, k) in zip(self.parts, states):
            p.Y.copy_(Y), p.memory.copy_(m), p.counts.copy_(c), p.status.copy_(st), p.k.copy_(k)
        self.t.copy_(t_saved)
        torch.cuda.synchronize(self.dev)
        with torch.cuda.graph(g, stream=s):
            self.enqueue_interval(s)
        torch.cuda.synchronize(self.dev)
        self.graph = g
        return g

    def run(self, intervals: int, graph: bool = True):
        if graph and self.graph is None:
            self.capture()
        for _ in range(int(intervals)):
            if graph:
                self.graph.replay()
            else:
                self.enqueue_interval()

    def reset(self, t0: float = 0.0):
        for p in self.parts:
            p.reset()
        self.t.fill_(float(t0))
