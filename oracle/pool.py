"""A pool of CPU workers for the CPU baseline (test/bench infrastructure).

Each worker runs the reference's own Algorithm(ROS3).solve when the reference
is installed in baseline/_ref, else the oracle's restatement of it. Each
spawned worker owns one group of 32 cells of the 210-species /
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


REFERENCE = ROOT / "baseline" / "_ref"


def reference_installed() -> bool:
    """True when the unmodified reference package is installed in
    baseline/_ref (pip install --target), so that its own code can be timed."""
    return (REFERENCE / "fastode" / "solvers.py").is_file()


def group_solver(wl):
    """(kind, step) for one group of the workload: step(Y, k, counts, mem)
    advances it by one interval with the reference's own Algorithm(ROS3).solve
    when it is installed (kind "reference"), else with the oracle's
    restatement of it (kind "port"); also returns fresh counts and memory."""
    if reference_installed():
        sys.path.insert(0, str(REFERENCE))
        from fastode import ROS3, Algorithm, Counts
        from fastode.chem import ChemSystem, Mechanism
        mech = Mechanism(wl.sm.species, wl.sm.reactions)
        alg = Algorithm(ROS3)

        def step(Y, k, counts, mem):
            return alg.solve(ChemSystem(mech, k), Y, wl.dt, wl.atol, wl.rtol, counts, mem)
        return "reference", step, Counts, alg.new_memory
    from oracle import rosenbrock as O
    alg = O.OAlgorithm(O.OROS3)

    def step(Y, k, counts, mem):
        return alg.solve(O.OChem(wl.sm.mech, k), Y, wl.dt, wl.atol, wl.rtol, counts, mem)
    return "port", step, O.OCounts, O.OMemory


def _worker(conn, group, n_cells):
    os.environ["OMP_NUM_THREADS"] = os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, str(ROOT))
    from fastode_gb300 import synthetic as syn

    wl = syn.plain_large(n_cells=n_cells, intervals=1).subset(slice(group * 32, group * 32 + 32))
    kind, step, new_counts, new_memory = group_solver(wl)

    def fresh():
        return wl.cells.Y0.copy(), new_memory(), new_counts(), 0

    Y, mem, counts, interval = fresh()
    conn.send(("ready", kind))
    while True:
        cmd = conn.recv()
        if cmd == "step":
            Y, st = step(Y, wl.k_at(interval), counts, mem)
            interval += 1
            conn.send(st)
        elif cmd == "reset":
            Y, mem, counts, interval = fresh()
            conn.send("ok")
        else:
            conn.send(tuple(counts.as_dict().values()))
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
        self.kinds = {c.recv()[1] for c in self.conns}
        self.kind = self.kinds.pop() if len(self.kinds) == 1 else "mixed"
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
