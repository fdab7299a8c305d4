"""Host-side checks (CPU only): tableaus, mechanism tables, the synthetic
generator, the C-ABI library's exports and its symbolic analysis."""
import ctypes
import re
import sys
from pathlib import Path

import numpy as np
import pytest

from golden_cases import CASES, load, mechanism_of, reactions_of

ROOT = Path(__file__).resolve().parents[1]
REFERENCE = Path("/root/reference")


@pytest.mark.parametrize("name", ["ros3", "rodas3"])
def test_order_conditions(name):
    # tests/test_fastode.py:21-31
    from fastode_gb300.tableaus import TABLEAUS
    tab = TABLEAUS[name]
    A, Gamma, b, bhat = tab.standard_form()
    beta = A + Gamma
    ap = A.sum(axis=1)
    bp = beta.sum(axis=1)
    assert abs(b.sum() - 1) < 1e-12
    assert abs(b @ bp - 0.5) < 1e-12
    assert abs(b @ ap ** 2 - 1 / 3) < 1e-12
    assert abs(b @ (beta @ bp) - 1 / 6) < 1e-12
    assert abs(bhat.sum() - 1) < 1e-12 and abs(bhat @ bp - 0.5) < 1e-12


def test_forcing_reuse_flags():
    # tests/test_fastode.py:39-41
    from fastode_gb300 import ROS3, RODAS3
    assert ROS3.new_forcing == [True, True, False]
    assert RODAS3.new_forcing == [True, False, True, True]


def test_quantize():
    # tests/test_fastode.py:89-93
    from fastode_gb300 import quantize
    for h in (1.0, 7.3, 33.0, 600.0, 900.0):
        q = quantize(h, 600.0)
        n = round(600.0 / q)
        assert abs(n * q - 600.0) < 1e-9 and h / 2 < q <= h or h >= 600.0


def test_counts_fields_match_device_order():
    from fastode_gb300.counts import COUNT_FIELDS, Counts
    c = Counts()
    assert tuple(c.as_dict().keys()) == COUNT_FIELDS
    c.add_row(range(13))
    assert c.calls == 12 and c.steps == 0


@pytest.mark.parametrize("case", CASES)
def test_generator_reproduces_fixture_inputs(case):
    """The seeded generator still yields the inputs the fixtures were made from."""
    from fastode_gb300 import synthetic as syn
    f = load(case)
    wl = syn.plain_small() if case == "ros3_20x40" else syn.plain_large(n_cells=64, intervals=4)
    species, reactions = reactions_of(f)
    assert reactions == wl.sm.reactions
    C = f["Y0"].shape[0]
    np.testing.assert_array_equal(wl.cells.Y0[:C], f["Y0"])
    for i in range(int(f["intervals"])):
        np.testing.assert_allclose(wl.k_at(i)[:C], f["k"][i], rtol=1e-15, atol=0)


@pytest.mark.skipif(not REFERENCE.exists(), reason="reference checkout not present")
@pytest.mark.parametrize("case", CASES)
def test_mechanism_tables_match_reference(case):
    """Mechanism builds the reference's react, S, pattern and GT map."""
    sys.path.insert(0, str(REFERENCE))
    from fastode.chem import Mechanism as RMech
    f = load(case)
    species, reactions = reactions_of(f)
    ours = mechanism_of(f)
    ref = RMech(species, reactions)
    assert np.array_equal(ours.react, ref.react)
    assert np.array_equal(ours.S, ref.S)
    assert np.array_equal(ours.pattern.rows, ref.pattern.rows)
    assert np.array_equal(ours.pattern.cols, ref.pattern.cols)
    ind, idx, val = ours.jac_csr()
    assert np.array_equal(ind, ref.GT.indptr) and np.array_equal(idx, ref.GT.indices)
    assert np.array_equal(val, ref.GT.data)


def declared_symbols():
    text = (ROOT / "include" / "fastode_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fo_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_library):
    lib = ctypes.CDLL(str(built_library))
    names = declared_symbols()
    assert "fo_solve" in names and "fo_analyze" in names
    for name in names:
        assert hasattr(lib, name), name
    from fastode_gb300 import _abi
    assert set(_abi.SIGNATURES) == set(names)


def structural_lu(n, rows, cols, perm):
    """Fill pattern and multiply-add count of a pivot-free dense elimination
    in the order perm, computed on booleans."""
    pos = np.empty(n, dtype=np.int64)
    pos[perm] = np.arange(n)
    A = np.zeros((n, n), dtype=bool)
    A[pos[rows], pos[cols]] = True
    A[np.arange(n), np.arange(n)] = True
    fma = 0
    for k in range(n):
        below = np.nonzero(A[k + 1:, k])[0] + k + 1
        right = np.nonzero(A[k, k + 1:])[0] + k + 1
        fma += len(below) * len(right)
        A[np.ix_(below, right)] = True
    return A, fma


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("ordering", ["natural", "min_degree", "min_fill", "auto", "refined"])
def test_symbolic_analysis_matches_dense_elimination(built_library, case, ordering):
    from fastode_gb300.plan import analyze
    mech = mechanism_of(load(case))
    info = analyze(mech, ordering)
    perm = info["perm"]
    assert sorted(perm.tolist()) == list(range(mech.n))
    A, fma = structural_lu(mech.n, mech.pattern.rows, mech.pattern.cols, perm)
    assert info["nnz_lu"] == int(A.sum())
    assert info["lu_fma"] == fma
    assert info["nnz_l"] == int(np.tril(A, -1).sum()) and info["nnz_u"] == int(np.triu(A, 1).sum())


def test_auto_ordering_is_the_cheapest(built_library):
    from fastode_gb300.plan import analyze
    mech = mechanism_of(load("ros3_210x500"))
    costs = {o: analyze(mech, o)["lu_fma"] for o in ("natural", "min_degree", "min_fill")}
    assert analyze(mech, "auto")["lu_fma"] <= min(costs.values())
    assert costs["min_degree"] < costs["natural"]


def test_refined_ordering_is_deterministic_and_cheaper(built_library):
    """The local search on the elimination order gives the same order on every
    call, and on the 210-species mechanism it removes well over a quarter of
    the greedy orders' LU FMAs."""
    from fastode_gb300.plan import analyze
    mech = mechanism_of(load("ros3_210x500"))
    a, b = analyze(mech, "refined"), analyze(mech, "refined")
    np.testing.assert_array_equal(a["perm"], b["perm"])
    greedy = min(analyze(mech, o)["lu_fma"] for o in ("natural", "min_degree", "min_fill"))
    assert a["lu_fma"] <= 0.7 * greedy, (a["lu_fma"], greedy)
    assert analyze(mech, "auto")["lu_fma"] == a["lu_fma"]


def test_analysis_rejects_bad_descriptors(built_library):
    from fastode_gb300 import _abi
    from fastode_gb300.chem import Mechanism
    from fastode_gb300.plan import _Desc
    mech = Mechanism(["A", "B"], [(["A"], [("B", 1.0)])])
    d = _Desc(mech)
    d.arrays["rows"][0] = 7              # out of range
    info = _abi.PlanInfo()
    rc = _abi.lib().fo_analyze(ctypes.byref(d.desc), 0, ctypes.byref(info), None)
    assert rc == -1
    assert b"out of range" in _abi.lib().fo_last_error()


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes structures of the binding have the offsets and sizes the C
    compiler gives the header's structs (compiled here with the host gcc)."""
    import shutil
    import subprocess
    from fastode_gb300 import _abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    structs = {"fo_options": _abi.Options, "fo_batch_desc": _abi.BatchDesc,
               "fo_mechanism_desc": _abi.MechanismDesc, "fo_plan_info": _abi.PlanInfo,
               "fo_gen_info": _abi.GenInfo, "fo_rate_law": _abi.RateLaw}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fastode_gb300.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{cname}.{field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert int(got[f"{cname}.{field}"]) == getattr(cls, field).offset, (cname, field)


def test_backward_euler_options_and_validation():
    """BackwardEuler keeps the reference's constructor defaults
    (fastode/solvers.py:423-427) and maps them onto fo_options."""
    from fastode_gb300 import BackwardEuler, _abi
    be = BackwardEuler()
    assert be.name == "backward-euler" and be.new_memory() is None
    o = be.options()
    assert o.loop == _abi.LOOPS["backward-euler"] and o.max_iterations == 11
    assert o.nreductions == 5 and list(o.reductions)[:5] == [0.5, 0.5, 0.5, 0.5, 0.1]
    assert o.small == 1.0e-40
    with pytest.raises(ValueError):
        BackwardEuler(reductions=(0.5, 0.0))
    with pytest.raises(ValueError):
        BackwardEuler(reductions=(0.5,) * 9)
    # the convergence test of fastode/solvers.py:432-437
    Y = np.array([[1.0, 1e-30]])
    atol = np.array([1e-12, 1e-12])
    assert be.converged(np.array([[1e-7, 1e-13]]), Y, atol, 1e-6)
    assert not be.converged(np.array([[1e-5, 0.0]]), Y, atol, 1e-6)
    assert not be.converged(np.array([[np.nan, 0.0]]), Y, atol, 1e-6)


def _write_descriptor(path, mech):
    from fastode_gb300.chem import mechanism_tables
    t = mechanism_tables(mech)
    arrays = [np.array([t["n"], t["R"], t["P"]], dtype=np.int64), np.asarray(t["react"], np.int64),
              np.asarray(t["s_indptr"], np.int32), np.asarray(t["s_idx"], np.int32), np.asarray(t["s_val"], np.float64),
              np.asarray(t["rows"], np.int64), np.asarray(t["cols"], np.int64),
              np.asarray(t["j_indptr"], np.int32), np.asarray(t["j_idx"], np.int32), np.asarray(t["j_val"], np.float64)]
    with open(path, "wb") as fh:
        for a in arrays:
            fh.write(np.int64(a.size).tobytes())
            fh.write(np.ascontiguousarray(a).tobytes())


@pytest.fixture(scope="module")
def compact_emulator(tmp_path_factory):
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    out = tmp_path_factory.mktemp("emu") / "compact_emulator"
    csrc = ROOT / "fast-ode-atmospheric-chem_gb300" / "csrc"
    subprocess.run([cxx, "-std=c++17", "-O2", f"-I{csrc}", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "compact_emulator.cpp"), str(csrc / "symbolic.cpp"), "-o", str(out)],
                   check=True)
    return out


@pytest.mark.parametrize("which", ["ros3_20x40", "ros3_210x500", "ts1", "dae", "60x40", "120x260", "1x1", "2x2", "3x4"])
def test_compact_tables_reproduce_the_plain_factorization(compact_emulator, tmp_path, which):
    """The compact variant's two-pass elimination stream and split solves,
    executed on the host over the tables the library builds, give the plain
    row-by-row factorization bit for bit and its solution to roundoff."""
    import subprocess
    from fastode_gb300 import synthetic as syn
    from golden_cases import table_mechanism
    if which.startswith("ros3"):
        mech = mechanism_of(load(which))
    elif which == "ts1":
        mech = table_mechanism(load("ts1_tier1_30s"))
    elif which == "dae":
        mech = syn.dae_constrained(n_cells=32, intervals=1).sm.mech
    elif which in ("1x1", "2x2", "3x4"):                 # empty and one-row halves
        n, r = (int(v) for v in which.split("x"))
        mech = syn.synthetic_mechanism(n, r, seed=1).mech
    else:
        mech = {"60x40": syn.batched_uneven(n_cells=96, intervals=1)[0],
                "120x260": syn.batched_uneven(n_cells=96, intervals=1)[1]}[which].sm.mech
    desc = tmp_path / "mech.bin"
    _write_descriptor(desc, mech)
    r = subprocess.run([str(compact_emulator), str(desc)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_large_mechanism_falls_back_from_the_stream_kernels(built_library):
    """A mechanism whose factor has more than 65,536 entries gets no packed
    streams: the plan reports the plain kernel's shared memory for the
    compact kernel too (the launch then runs the plain loops), and the
    ordering search stays within its operation budget."""
    import time
    from fastode_gb300 import synthetic as syn
    from fastode_gb300.plan import analyze
    sm = syn.synthetic_mechanism(1000, 2500, seed=5)
    t0 = time.perf_counter()
    info = analyze(sm.mech)
    assert time.perf_counter() - t0 < 30.0
    assert info["nnz_lu"] > 65536
    assert info["compact_smem_doubles_per_cell"] == info["smem_doubles_per_cell"]


def _gen_check(mech, link):
    from fastode_gb300 import _abi
    from fastode_gb300.plan import _Desc
    d = _Desc(mech)
    info = _abi.GenInfo()
    rc = _abi.lib().fo_generate_check(ctypes.byref(d.desc), _abi.ORDERINGS["auto"], int(link), ctypes.byref(info))
    return rc, info.as_dict(), _abi.lib().fo_last_error().decode()


def test_generated_code_links_with_the_integrator(built_library):
    """The generated variant of a small mechanism: its PTX is generated (the
    generator checks its multiply-add count against the symbolic analysis)
    and links with the library's relocatable integrator (nvJitLink, no
    device needed)."""
    from fastode_gb300 import synthetic as syn
    rc, info, err = _gen_check(syn.plain_small().sm.mech, link=True)
    assert rc == 0, err
    assert info["ptx_bytes"] > 0 and info["cubin_bytes"] > 0 and info["tile"] == 6


def test_generated_factorization_in_pieces_links(built_library):
    """A mechanism whose factorization is generated as several separately
    compiled functions (120 species / 260 reactions: 49,079 multiply-adds,
    about 100,000 instructions, three pieces of whole row blocks) links with
    the integrator: the pieces, the dispatching fo_gen_factor and the calls
    between them are valid for ptxas (nvJitLink, no device needed)."""
    from fastode_gb300 import synthetic as syn
    sm = syn.synthetic_mechanism(120, 260, 13, third_body_fraction=0.1)
    rc, info, err = _gen_check(sm.mech, link=True)
    assert rc == 0, err
    assert info["cubin_bytes"] > 0


@pytest.mark.parametrize("case", CASES)
def test_generated_code_covers_every_update(built_library, case):
    """Generation alone (no link) for the fixtures' mechanisms, the 210/500
    one included: one fused multiply-add per update of the symbolic LU."""
    rc, info, err = _gen_check(mechanism_of(load(case)), link=False)
    assert rc == 0, err
    assert info["ptx_bytes"] > 0


def test_lockstep_option_reaches_fo_options():
    """Algorithm(lockstep=...) sets fo_options.lockstep (the rounds of the
    generated kernel are on by default, a speed choice only); the other
    step loops keep the Algorithm value they inherit."""
    from fastode_gb300 import Algorithm, RestartingLoop
    assert Algorithm().options().lockstep == 1
    assert Algorithm(lockstep=False).options().lockstep == 0
    assert RestartingLoop().options().lockstep == 1
