"""The oracle's hand-written adjoint of the differentiable rollout (oracle/diff_oracle.inc), checked
without a GPU: against torch float64 autograd of an independent restatement of the rollout
(oracle/torch_rollout.py) and against FP64 central finite differences, on a small lattice with a
capsule pressing into it.  The CUDA adjoint is compared with this oracle in the GPU tests."""
import ctypes

import numpy as np
import pytest
import torch

from diff_cases import YOUNG, Case, bind_oracle, oracle_adjoint, oracle_rollout, torch_rollout_module


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.fixture(scope="module")
def case():
    return Case()


@pytest.fixture
def f64_session(oracle_libs, case):
    """One session per test: a library holds a single process-global session."""
    s = case.session(oracle_libs[1])
    dll = bind_oracle(s.dll)
    assert dll.ORC_DiffBegin(YOUNG, case.every, case.frames) == 0
    yield s, dll
    dll.ORC_DiffEnd()
    s.close()


def test_rollout_moves_and_contacts(f64_session, case):
    s, dll = f64_session
    theta = case.theta(s.tet_count)
    free = oracle_rollout(dll, case, theta, None)
    pressed = oracle_rollout(dll, case, theta, case.path)
    assert np.isfinite(pressed).all()
    assert np.abs(free - case.grid.positions).max() > 1e-4          # gravity sag
    assert np.abs(pressed - free).max() > 1e-3                      # the capsule pushes nodes


def test_adjoint_matches_autograd_fp64(f64_session, case):
    s, dll = f64_session
    tr = torch_rollout_module()
    topo = tr.export_topology(dll)
    theta = case.theta(s.tet_count).astype(np.float64)
    weights = np.random.default_rng(1).standard_normal((case.n, 3))
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    pa = torch.tensor(case.path.astype(np.float64), requires_grad=True)
    origin = case.grid.positions.astype(np.float64)
    x = tr.rollout(topo, origin, np.zeros_like(origin), th, pa, case.radius, case.dt, case.substeps, case.frames, YOUNG)
    final = oracle_rollout(dll, case, theta, case.path)
    assert np.abs(x.detach().numpy() - final).max() < 1e-10          # the two FP64 rollouts agree
    (x * torch.tensor(weights)).sum().backward()
    adj = oracle_adjoint(dll, case, weights, s.tet_count)
    assert rel(adj["theta"], th.grad.numpy()) < 1e-8
    assert rel(adj["path"], pa.grad.numpy()) < 1e-8
    assert np.abs(th.grad.numpy()).max() > 0 and np.abs(pa.grad.numpy()).max() > 0


def test_adjoint_matches_central_differences_fp64(f64_session, case):
    s, dll = f64_session
    theta = case.theta(s.tet_count).astype(np.float64)
    path = case.path.astype(np.float64)
    rng = np.random.default_rng(2)
    weights = rng.standard_normal((case.n, 3))
    oracle_rollout(dll, case, theta, path)
    adj = oracle_adjoint(dll, case, weights, s.tet_count)
    eps = 1e-5
    fd, an = [], []
    for _ in range(6):
        dt_, dp = rng.standard_normal(theta.shape), rng.standard_normal(path.shape) * 0.05
        up = (oracle_rollout(dll, case, theta + eps * dt_, path + eps * dp) * weights).sum()
        dn = (oracle_rollout(dll, case, theta - eps * dt_, path - eps * dp) * weights).sum()
        fd.append((up - dn) / (2 * eps))
        an.append((adj["theta"] * dt_).sum() + (adj["path"] * dp).sum())
    assert rel(an, fd) < 1e-6, (an, fd)


def test_rest_shape_and_origin_adjoints_match_autograd(oracle_libs, case):
    """Rest-length and origin-state adjoints against autograd of the same restatement.  The origin
    is a deformed, moving state (three plain frames of sag): at the undeformed rest state every tet
    sits at the kink of C_D = sqrt(max(q, 1e-12)), where position derivatives are not defined."""
    s = case.session(oracle_libs[1])
    try:
        dll = bind_oracle(s.dll)
        for _ in range(3):
            s.step()
        origin_pos = np.zeros((case.n, 3))
        origin_vel = np.zeros((case.n, 3))
        assert s.dll.ORC_GetCornerPos64(origin_pos.ctypes.data_as(ctypes.c_void_p)) == 0
        assert s.dll.ORC_GetVelocities64(origin_vel.ctypes.data_as(ctypes.c_void_p)) == 0
        assert dll.ORC_DiffBegin(YOUNG, case.every, case.frames) == 0
        tr = torch_rollout_module()
        topo = tr.export_topology(dll)
        theta = case.theta(s.tet_count).astype(np.float64)
        weights = np.random.default_rng(4).standard_normal((case.n, 3))
        oracle_rollout(dll, case, theta, case.path)
        adj = oracle_adjoint(dll, case, weights, s.tet_count, rest=True, origin=True)
        origin = torch.tensor(origin_pos, requires_grad=True)
        velocity = torch.tensor(origin_vel, requires_grad=True)
        rest = torch.tensor(topo["eRest"], requires_grad=True)
        x = tr.rollout(dict(topo, eRest=rest), origin, velocity, torch.tensor(theta), torch.tensor(case.path.astype(np.float64)),
                       case.radius, case.dt, case.substeps, case.frames, YOUNG)
        (x * torch.tensor(weights)).sum().backward()
        assert rel(adj["origin"][0], origin.grad.numpy()) < 1e-7
        assert rel(adj["origin"][1], velocity.grad.numpy()) < 1e-7
        # the oracle reports rest-length adjoints at the owner slot 6p + s of each edge
        nbr = case.grid.neighbors
        owner = []
        for i, j in topo["eIJ"]:
            slots = np.nonzero(nbr[i] == j)[0]
            owner.append(6 * i + slots[0] if len(slots) else -1)
        owner = np.array(owner)
        mask = owner >= 0
        assert mask.sum() > 0.9 * len(mask)
        assert rel(adj["rest_length"].reshape(-1)[owner[mask]], rest.grad.numpy()[mask]) < 1e-7
        dll.ORC_DiffEnd()
    finally:
        s.close()


def test_fp32_adjoint_close_to_fp64(oracle_libs, case):
    """FP32 against FP64 with the compliance read relative to 1e-6/Pa (Young's moduli 0.6-60 kPa):
    strains are then well above FP32 rounding of the invariants, so the deviatoric projection's
    direction, and with it the adjoint, is resolved in FP32."""
    grads = []
    for lib in oracle_libs:
        s = case.session(lib)
        try:
            dll = bind_oracle(s.dll)
            assert dll.ORC_DiffBegin(1e6, case.every, case.frames) == 0
            theta = case.theta(s.tet_count)
            oracle_rollout(dll, case, theta, case.path)
            grads.append(oracle_adjoint(dll, case, np.ones((case.n, 3)), s.tet_count))
            dll.ORC_DiffEnd()
        finally:
            s.close()
    assert rel(grads[0]["theta"], grads[1]["theta"]) < 1e-3
    assert rel(grads[0]["path"], grads[1]["path"]) < 1e-3
