"""fo_solve_static, the entry point for callers that cannot allocate device
memory (a host model whose memory pool owns the device, a time step that cannot
afford cudaMalloc's implicit synchronization): called through the C-ABI twice
in a row, it must give what fo_solve with a caller-provided workspace gives on
the same inputs. The file is named to run last, and it sets up everything it
uses itself, so it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from golden_cases import load, mechanism_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["ros3_20x40", "ros3_210x500"])
def test_static_scratch_matches_workspace_entry_point(cuda, case):
    from fastode_gb300 import Algorithm, _abi
    from fastode_gb300.batch import group_offsets
    from fastode_gb300.plan import plan_for
    torch = cuda
    f = load(case)
    mech = mechanism_of(f)
    plan = plan_for(mech)
    lib = _abi.lib()
    Cc, n = f["Y0"].shape
    offs = torch.from_numpy(group_offsets(Cc, 32)).cuda()
    G = len(offs) - 1
    atol = torch.from_numpy(f["atol"]).cuda()
    opts = plan.options_for(Algorithm(), 32)     # the default (generated) variant
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def state():
        return dict(Y=torch.from_numpy(np.ascontiguousarray(f["Y0"].T)).cuda(),
                    mem=torch.zeros((G, 3), dtype=torch.float64, device="cuda"),
                    cnt=torch.zeros((G, 13), dtype=torch.int64, device="cuda"),
                    st=torch.zeros(G, dtype=torch.int32, device="cuda"))

    a, b = state(), state()
    ws = torch.empty(plan.workspace_bytes(G, 32), dtype=torch.uint8, device="cuda")
    for i in range(2):                                   # two calls in a row
        k = torch.from_numpy(np.ascontiguousarray(f["k"][i].T)).cuda()
        rc = lib.fo_solve(plan.handle, C.byref(opts), G, offs.data_ptr(), 32, a["Y"].data_ptr(), 1, Cc,
                          k.data_ptr(), 1, Cc, atol.data_ptr(), float(f["rtol"]), float(f["dt"]),
                          a["mem"].data_ptr(), a["cnt"].data_ptr(), a["st"].data_ptr(), ws.data_ptr(), ws.numel(),
                          0, None, 0, None, stream)
        _abi.check(rc, "fo_solve")
        rc = lib.fo_solve_static(plan.handle, C.byref(opts), G, offs.data_ptr(), 32, b["Y"].data_ptr(), 1, Cc,
                                 k.data_ptr(), 1, Cc, atol.data_ptr(), float(f["rtol"]), float(f["dt"]),
                                 b["mem"].data_ptr(), b["cnt"].data_ptr(), b["st"].data_ptr(), stream)
        _abi.check(rc, "fo_solve_static")
        torch.cuda.synchronize()
        Ya, Yb = a["Y"].cpu().numpy(), b["Y"].cpu().numpy()
        assert np.all(np.abs(Yb - Ya) <= 1e-10 * np.maximum(np.abs(Ya), 1e-14)), i
        np.testing.assert_array_equal(b["cnt"].cpu().numpy(), a["cnt"].cpu().numpy())
        np.testing.assert_array_equal(b["st"].cpu().numpy(), a["st"].cpu().numpy())
        # all of the controller memory: h_next, and the error and step history
        # that the next interval's H211b factor consumes
        np.testing.assert_array_equal(b["mem"].cpu().numpy(), a["mem"].cpu().numpy())


def _tiled_subset(copies):
    """The 210/500 parity subset (eight groups) repeated `copies` times: inputs
    of copies * 8 groups, with the fixture's k of every interval."""
    f = load("ros3_210x500_subset")
    Y0 = np.tile(f["Y0"], (copies, 1))
    ks = []
    for i in range(int(f["intervals"])):
        k = np.array(f["k0"], copy=True)
        k[:, f["photo"]] = f["J"][None, :] * f["f"][i][:, None]
        ks.append(np.tile(k, (copies, 1)))
    return f, Y0, ks


def test_static_scratch_with_more_groups_than_slots(cuda):
    """24 groups of the 210/500 mechanism against the seven slots that fit in
    the static array: the slots take groups from the device queue in turn, and
    each reused slot still starts every group from its own inputs. Four
    intervals in a row (the controller memory of one interval feeds the next),
    then a call with another group count; everything fo_solve gives with its
    own workspace, bit for bit (the same kernel on the same inputs)."""
    from fastode_gb300 import Algorithm, _abi
    from fastode_gb300.batch import group_offsets
    from fastode_gb300.plan import plan_for
    torch = cuda
    f, Y0, ks = _tiled_subset(3)
    plan = plan_for(mechanism_of(f))
    slot = plan.workspace_bytes(2, 32) - plan.workspace_bytes(1, 32)
    lib = _abi.lib()
    atol = torch.from_numpy(f["atol"]).cuda()
    opts = plan.options_for(Algorithm(), 32)     # the default (generated) variant
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def state(Yh):
        G = Yh.shape[0] // 32
        return dict(Y=torch.from_numpy(np.ascontiguousarray(Yh.T)).cuda(), G=G, C=Yh.shape[0],
                    offs=torch.from_numpy(group_offsets(Yh.shape[0], 32)).cuda(),
                    mem=torch.zeros((G, 3), dtype=torch.float64, device="cuda"),
                    cnt=torch.zeros((G, 13), dtype=torch.int64, device="cuda"),
                    st=torch.zeros(G, dtype=torch.int32, device="cuda"))

    def call(entry, s, k, ws=None):
        args = [plan.handle, C.byref(opts), s["G"], s["offs"].data_ptr(), 32, s["Y"].data_ptr(), 1, s["C"],
                k.data_ptr(), 1, s["C"], atol.data_ptr(), float(f["rtol"]), float(f["dt"]),
                s["mem"].data_ptr(), s["cnt"].data_ptr(), s["st"].data_ptr()]
        if entry == "fo_solve":
            args += [ws.data_ptr(), ws.numel(), 0, None, 0, None, stream]
        else:
            args += [stream]
        _abi.check(getattr(lib, entry)(*args), entry)

    def same(a, b):
        torch.cuda.synchronize()
        for key in ("Y", "mem", "cnt", "st"):
            np.testing.assert_array_equal(b[key].cpu().numpy(), a[key].cpu().numpy(), err_msg=key)

    a, b = state(Y0), state(Y0)
    assert a["G"] >= 3 * ((32 << 20) // slot), (a["G"], slot)
    ws = torch.empty(plan.workspace_bytes(a["G"], 32), dtype=torch.uint8, device="cuda")
    for i in range(4):
        k = torch.from_numpy(np.ascontiguousarray(ks[i][: a["C"]].T)).cuda()
        call("fo_solve", a, k, ws)
        call("fo_solve_static", b, k)
        same(a, b)
    # the next call has another group count (nine groups: more than the slots
    # again, and not a multiple of them)
    a2, b2 = state(Y0[: 9 * 32]), state(Y0[: 9 * 32])
    for i in range(2):
        k = torch.from_numpy(np.ascontiguousarray(ks[i][: a2["C"]].T)).cuda()
        call("fo_solve", a2, k, ws)
        call("fo_solve_static", b2, k)
        same(a2, b2)
