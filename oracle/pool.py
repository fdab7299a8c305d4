"""A pool of oracle workers for the CPU baseline (test/bench infrastructure).

Each spawned worker owns one group of 32 cells of the 210-species /
500-reaction synthetic workload and its controller memory, as the reference's
scenario loop keeps one Memory per group (fastode/ts1.py:196-222); a step
advances every worker's group by one interval. BLAS runs one thread per
process, as the reference's experiment pool pins it
(experiments/ts1_experiments.py:22-24, 158-163).
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _worker(conn, group, n_cells):
    os.environ["OMP_NUM_THREADS"] = os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, str(ROOT))
    from fastode_gb300 import synthetic as syn
    from oracle import rosenbrock as O

    wl = syn.plain_large(n_cells=n_cells, intervals=1).subset(slice(group * 32, group * 32 + 32))

    def fresh():
        return wl.cells.Y0.copy(), O.OMemory(), O.OCounts(), 0

    Y, mem, counts, interval = fresh()
    alg = O.OAlgorithm(O.OROS3)
    conn.send("ready")
    while True:
        cmd = conn.recv()
        if cmd == "step":
            k = wl.k_at(interval)
            Y, st = alg.solve(O.OChem(wl.sm.mech, k), Y, wl.dt, wl.atol, wl.rtol, counts, mem)
            interval += 1
            conn.send(st)
        elif cmd == "reset":
            Y, mem, counts, interval = fresh()
            conn.send("ok")
        else:
            conn.send(counts.as_tuple())
            return


class GroupPool:
    def __init__(self, ctx, workers, n_cells):
        self.ctx = ctx
        self.workers = workers
        self.n_cells = n_cells

    def __enter__(self):
        self.conns, self.procs = [], []
        for g in range(self.workers):
            a, b = self.ctx.Pipe()
            p = self.ctx.Process(target=_worker, args=(b, g % (self.n_cells // 32), self.n_cells), daemon=True)
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        for c in self.conns:
            c.recv()
        return self

    def _all(self, cmd):
        for c in self.conns:
            c.send(cmd)
        return [c.recv() for c in self.conns]

    def step(self):
        return self._all("step")

    def reset(self):
        return self._all("reset")

    def __exit__(self, *a):
        try:
            self._all("stop")
        finally:
            for p in self.procs:
                p.join(timeout=10)
                if p.is_alive():
                    p.terminate()
