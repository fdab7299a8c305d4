"""The discrete adjoint on the GPU (new: the reference has no sensitivities),
checked against the host FP64 tangent-linear (complex step through the
oracle's fixed-step map) and against central finite differences of the
device's own fixed-step replay (h = 1e-6), with the accepted step sizes of the
forward run held fixed."""
import numpy as np
import pytest

from golden_cases import load, mechanism_of

pytestmark = pytest.mark.gpu


def record(cuda, case="ros3_20x40", intervals=5, groups=2):
    from fastode_gb300.adjoint import forward_record
    torch = cuda
    f = load(case)
    mech = mechanism_of(f)
    C = 32 * groups
    ks = [torch.from_numpy(np.ascontiguousarray(f["k"][i][:C].T)).cuda() for i in range(intervals)]
    traj = forward_record(mech, f["Y0"][:C], lambda i: ks[i], float(f["dt"]), f["atol"], float(f["rtol"]),
                          intervals)
    return f, mech, traj, ks


def host_steps(traj, g, i):
    p = traj.step_ptr[i].cpu().numpy()
    s = traj.steps[i].cpu().numpy()
    return s[p[g]:p[g + 1]].tolist()


def test_replay_reproduces_the_forward_run(cuda):
    from fastode_gb300.adjoint import replay
    f, mech, traj, ks = record(cuda)
    Y = replay(traj)
    np.testing.assert_array_equal(Y.cpu().numpy(), traj.batch.Y.cpu().numpy())


@pytest.mark.parametrize("case", ["ros3_20x40", "ros3_210x500"])
def test_adjoint_matches_host_tangent_linear(cuda, case):
    """<lam_end, dY_end> from the host tangent-linear equals
    <lam_0, dY0> + <dL/dlog k, dlog k> from the device adjoint."""
    from fastode_gb300.adjoint import adjoint
    from oracle import rosenbrock as O
    torch = cuda
    intervals = 4 if case == "ros3_20x40" else 2
    f, mech, traj, ks = record(cuda, case, intervals=intervals, groups=1)
    C = traj.batch.C
    rng = np.random.default_rng(1)
    Y0 = f["Y0"][:C]
    dY0 = Y0 * rng.standard_normal(Y0.shape)
    dth = rng.standard_normal(mech.R)
    lam_end = rng.standard_normal((C, mech.n)) / np.maximum(np.abs(traj.batch.state()), 1e-14)
    lam0, thbar = adjoint(traj, torch.from_numpy(np.ascontiguousarray(lam_end.T)).cuda())
    lam0 = lam0.cpu().numpy().T
    thbar = thbar.cpu().numpy()                    # (R, C)
    adj = np.sum(lam0 * dY0) + np.sum(thbar.sum(axis=1) * dth)
    k_host = [f["k"][i][:C] for i in range(intervals)]
    tl, Yend = O.tangent_linear(mech, Y0, dY0, k_host, dth, [host_steps(traj, 0, i) for i in range(intervals)])
    ref = np.sum(lam_end * tl)
    scale = np.sum(np.abs(lam_end * tl))
    assert abs(adj - ref) <= 1e-8 * scale, (adj, ref, scale)


def test_adjoint_matches_central_differences(cuda):
    """Directional derivatives of L = sum(w * Y_end) by central differences
    (h = 1e-6) of the device's fixed-step replay, on random directions."""
    from fastode_gb300.adjoint import adjoint, replay
    torch = cuda
    f, mech, traj, ks = record(cuda, intervals=3)
    C = traj.batch.C
    rng = np.random.default_rng(2)
    Yend = traj.batch.Y.cpu().numpy()             # (n, C)
    w = rng.standard_normal(Yend.shape) / np.maximum(np.abs(Yend), 1e-14)
    lam0, thbar = adjoint(traj, torch.from_numpy(w).cuda())
    g_y = lam0.cpu().numpy()
    g_th = thbar.cpu().numpy().sum(axis=1)
    Y0 = traj.checkpoints[0]
    h = 1e-6
    for d in range(4):
        dY = torch.from_numpy(Y0.cpu().numpy() * rng.standard_normal(Y0.shape)).cuda()
        dth = rng.standard_normal(mech.R)

        def L(sign):
            kk = [k * torch.from_numpy(np.exp(sign * h * dth)).cuda()[:, None] for k in ks]
            return float(np.sum(w * replay(traj, Y0 + sign * h * dY, kk).cpu().numpy()))

        fd = (L(1.0) - L(-1.0)) / (2 * h)
        adj = float(np.sum(g_y * dY.cpu().numpy()) + np.sum(g_th * dth))
        assert abs(adj - fd) <= 1e-6 * max(abs(fd), 1e-300) + 1e-9 * np.sum(np.abs(w)), (d, adj, fd)


def test_autograd_function(cuda):
    """torch.autograd through fastode_gb300.adjoint.integrate gives the
    adjoint's gradients."""
    from fastode_gb300.adjoint import integrate
    torch = cuda
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    C = 32
    ks = [torch.from_numpy(np.ascontiguousarray(f["k"][i][:C].T)).cuda() for i in range(3)]
    Y0 = torch.from_numpy(f["Y0"][:C].copy()).cuda().requires_grad_(True)
    theta = torch.zeros(mech.R, dtype=torch.float64, device="cuda", requires_grad=True)
    spec = dict(mech=mech, base=ks, dt=float(f["dt"]), atol=f["atol"], rtol=float(f["rtol"]))
    Y = integrate(Y0, theta, spec)
    target = (Y.detach() * 1.1).clamp_min(1e-30)
    a = 1e-14
    loss = ((torch.log(Y + a) - torch.log(target + a)) ** 2).sum()
    loss.backward()
    assert Y0.grad is not None and theta.grad is not None
    assert torch.isfinite(Y0.grad).all() and torch.isfinite(theta.grad).all()
    assert float(theta.grad.abs().sum()) > 0.0


def host_proj_steps(traj, g, i):
    p = traj.proj_ptr[i].cpu().numpy()
    s = traj.proj_steps[i].cpu().numpy()
    return s[p[g]:p[g + 1]].tolist()


def test_constrained_rodas3_adjoint(cuda):
    """RODAS3 with ten algebraic species (mass 0, quasi-steady state): the
    constrained synthetic workload's 32 cells over its four 60 s intervals.
    Every call starts with the projection onto the constraints
    (fastode/solvers.py:100-178), which here applies Newton updates in every
    interval; the adjoint differentiates those updates (with the forward
    run's line-search steps held fixed) as well as the RODAS3 steps.
    Gradients with respect to the log rate constants and the state against
    the oracle's tangent-linear (complex step through the same fixed
    projection updates and steps, mass matrix included) and against central
    differences of the device's replay, which reproduces the forward run."""
    from fastode_gb300 import Algorithm, RODAS3
    from fastode_gb300.adjoint import adjoint, forward_record, replay
    from oracle import rosenbrock as O
    torch = cuda
    f = load("rodas3_dae_160x340")
    mech = mechanism_of(f)
    mass = f["mass"]
    dt, rtol = float(f["dt"]), float(f["rtol"])
    intervals = int(f["intervals"])
    ks = [torch.from_numpy(np.ascontiguousarray(f["k"][i].T)).cuda() for i in range(intervals)]
    Y0 = f["Y0"]
    traj = forward_record(mech, Y0, lambda i: ks[i], dt, f["atol"], rtol, intervals, algorithm=Algorithm(RODAS3),
                          mass=mass)
    assert all(s == ["converged"] for s in traj.statuses)
    proj = [host_proj_steps(traj, 0, i) for i in range(intervals)]
    assert sum(len(p) for p in proj) > 0, proj                     # the projection does move the state
    np.testing.assert_array_equal(replay(traj).cpu().numpy(), traj.batch.Y.cpu().numpy())

    rng = np.random.default_rng(5)
    dY0 = Y0 * rng.standard_normal(Y0.shape)
    dth = rng.standard_normal(mech.R)
    Yend = traj.batch.state()
    lam_end = rng.standard_normal(Yend.shape) / np.maximum(np.abs(Yend), 1e-14)
    lam0, thbar = adjoint(traj, torch.from_numpy(np.ascontiguousarray(lam_end.T)).cuda())
    g_y, g_th = lam0.cpu().numpy().T, thbar.cpu().numpy().sum(axis=1)
    adj = np.sum(g_y * dY0) + np.sum(g_th * dth)
    steps = [host_steps(traj, 0, i) for i in range(intervals)]
    tl, Yo = O.tangent_linear(mech, Y0, dY0, [f["k"][i] for i in range(intervals)], dth, steps,
                              tab=O.ORODAS3, mass=mass, proj_list=proj)
    ref = np.sum(lam_end * tl)
    assert abs(adj - ref) <= 1e-8 * np.sum(np.abs(lam_end * tl)), (adj, ref)

    h = 1e-6
    Y0d = traj.checkpoints[0]
    for d in range(3):
        dth = rng.standard_normal(mech.R)

        def L(sign):
            kk = [k * torch.from_numpy(np.exp(sign * h * dth)).cuda()[:, None] for k in traj.ks]
            return float(np.sum(lam_end.T * replay(traj, Y0d, kk).cpu().numpy()))

        fd = (L(1.0) - L(-1.0)) / (2 * h)
        adj = float(np.sum(g_th * dth))
        assert abs(adj - fd) <= 1e-6 * max(abs(fd), 1e-300) + 1e-9 * np.sum(np.abs(lam_end)), (d, adj, fd)
