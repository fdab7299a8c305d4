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
    opts = Algorithm().options()
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
        np.testing.assert_array_equal(b["mem"].cpu().numpy()[:, 0], a["mem"].cpu().numpy()[:, 0])
