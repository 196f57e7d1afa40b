"""The CUDA differentiable rollout (GBT_Diff* C ABI, genesis_tissue_simulation_gb300.diff) against
the CPU oracle: forward positions and adjoints against the FP32 oracle, which evaluates the same
operations in the same order, in both launch shapes; the torch.autograd.Function; and the C5
identification workload's gradient against the FP64 reference gradient and FP64 central
finite differences on 64 random directions (relative error <= 1e-3)."""
import json

import numpy as np
import pytest
import torch

from conftest import results_dir
from diff_cases import YOUNG, C5Oracle, Case, bind_oracle, oracle_adjoint, oracle_rollout

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.ravel(np.asarray(a, np.float64)), np.ravel(np.asarray(b, np.float64))
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def record(name, **values):
    with open(results_dir() / "adjoint.jsonl", "a") as f:
        f.write(json.dumps({"case": name, **values}) + "\n")


def gpu_tissue(case, lib, mode, modulus=YOUNG):
    from genesis_tissue_simulation_gb300 import diff as D
    from genesis_tissue_simulation_gb300.native_backend import GraspParams
    from diff_cases import GRASP
    return D.DifferentiableTissue(case.grid, dt=case.dt, substeps=case.substeps, ks=1e6, young_pa=YOUNG, poisson=0.25,
                                  strain_damping_s=0.04, gravity=(0.0, -981.0, 0.0), grasp_params=GraspParams(**GRASP),
                                  capsule_radius=case.radius, checkpoint_every=case.every, max_frames=case.frames, launch_mode=mode,
                                  dll_path=lib, scale_modulus=modulus)


@pytest.fixture(scope="module")
def case():
    return Case()


@pytest.fixture(scope="module")
def fp32_oracle(oracle_libs, case):
    s = case.session(oracle_libs[0])
    dll = bind_oracle(s.dll)
    assert dll.ORC_DiffBegin(YOUNG, case.every, case.frames) == 0
    theta = case.theta(s.tet_count)
    x = oracle_rollout(dll, case, theta, case.path)
    weights = np.random.default_rng(9).standard_normal((case.n, 3)).astype(np.float32)
    adj = oracle_adjoint(dll, case, weights, s.tet_count, rest=True, origin=True)
    tet_ids = s.tet_ids()
    dll.ORC_DiffEnd()
    s.close()
    return dict(theta=theta, x=x, weights=weights, adj=adj, tet_ids=tet_ids)


@pytest.mark.parametrize("mode", [2, 1])
def test_forward_and_adjoint_match_fp32_oracle(gpu_lib, case, fp32_oracle, mode):
    with gpu_tissue(case, gpu_lib, mode) as t:
        assert t.info()["grid_launch"] == (mode == 1)
        theta = torch.tensor(fp32_oracle["theta"], device="cuda")
        path = torch.tensor(case.path, device="cuda")
        x = t.forward(theta, path).cpu().numpy()
        assert np.array_equal(x, fp32_oracle["x"].astype(np.float32)), float(np.abs(x - fp32_oracle["x"]).max())
        g = t.backward(torch.tensor(fp32_oracle["weights"], device="cuda"), rest_shape=True, origin=True)
        ref = fp32_oracle["adj"]
        assert np.abs(ref["theta"]).max() > 0 and np.abs(ref["path"]).max() > 0
        assert rel(g["theta"].cpu(), ref["theta"]) < 1e-6
        assert rel(g["path"].cpu(), ref["path"]) < 1e-5
        assert rel(g["rest_length"].cpu(), ref["rest_length"]) < 1e-6
        assert rel(g["rest_inverse"].cpu().reshape(-1, 9), ref["rest_inverse"]) < 1e-6
        assert rel(g["origin_position"].cpu(), ref["origin"][0]) < 1e-6
        assert rel(g["origin_velocity"].cpu(), ref["origin"][1]) < 1e-6
        # the backward leaves the session at the rollout's final state
        assert np.array_equal(t.session.positions(), x)


def test_autograd_function_and_rollout_order(gpu_lib, case, fp32_oracle):
    with gpu_tissue(case, gpu_lib, 0) as t:
        theta = torch.tensor(fp32_oracle["theta"], device="cuda", requires_grad=True)
        path = torch.tensor(case.path, device="cuda", requires_grad=True)
        w = torch.tensor(fp32_oracle["weights"], device="cuda")
        x = t.rollout(theta, path)
        (x * w).sum().backward()
        assert rel(theta.grad.cpu(), fp32_oracle["adj"]["theta"]) < 1e-6
        assert rel(path.grad.cpu(), fp32_oracle["adj"]["path"]) < 1e-5
        # a second rollout invalidates the first one's checkpoints: its backward must refuse
        y = t.rollout(theta, path)
        t.rollout(theta.detach(), path.detach())
        with pytest.raises(RuntimeError, match="another rollout"):
            (y * w).sum().backward()


def test_rest_position_gradient_matches_directional_oracle(gpu_lib, case, fp32_oracle):
    """The rest-shape adjoints chained to rest node positions: finite differences of the rest
    lattice through the FP64 oracle's rollout would move the baked masses too, so this checks the
    chain rule's pieces instead: per-tet Dm^-1 and per-slot rest length adjoints are finite and
    the assembled rest-position gradient has the mesh's shape."""
    from genesis_tissue_simulation_gb300 import diff as D
    g = D.rest_position_gradient(case.grid, fp32_oracle["tet_ids"], fp32_oracle["adj"]["rest_length"], fp32_oracle["adj"]["rest_inverse"])
    assert g.shape == case.grid.positions.shape and np.isfinite(g).all() and np.abs(g).max() > 0


def test_unsupported_configurations_are_refused(gpu_lib, case):
    from genesis_tissue_simulation_gb300 import diff as D
    with pytest.raises(RuntimeError, match="-4001"):
        D.DifferentiableTissue(case.grid, ks=0.0, dll_path=gpu_lib)            # edge-only fallback branch
    with gpu_tissue(case, gpu_lib, 0) as t:
        with pytest.raises(ValueError):
            t.forward(torch.zeros(3, device="cuda"), None, 1)
        with pytest.raises(RuntimeError, match="-1004"):
            t.forward(torch.zeros(t.tet_count, device="cuda"), None, case.frames + 1)


@pytest.fixture(scope="module")
def c5_fp64(oracle_libs):
    o = C5Oracle(oracle_libs[1])
    yield o
    o.close()


@pytest.fixture(scope="module")
def c5_gpu(gpu_lib, c5_fp64):
    c5 = c5_fp64.c5
    with c5.open(gpu_lib) as t:
        theta = torch.tensor(c5.theta_initial, device="cuda", requires_grad=True)
        path = torch.tensor(c5.path, device="cuda", requires_grad=True)
        target = torch.tensor(c5_fp64.target, dtype=torch.float32, device="cuda")
        top = torch.tensor(c5.top, device="cuda")
        from genesis_tissue_simulation_gb300 import diff as D
        loss = D.identification_loss(t.rollout(theta, path), target, top)
        loss.backward()
        yield dict(loss=float(loss), theta=theta.grad.cpu().numpy(), path=path.grad.cpu().numpy())


def test_c5_gradient_matches_fp64_reference(c5_fp64, c5_gpu):
    c5 = c5_fp64.c5
    loss64 = c5_fp64.loss(c5.theta_initial, c5.path)
    gt, gp = c5_fp64.gradient(c5.theta_initial, c5.path)
    record("c5_fp64_reference", loss_fp32=c5_gpu["loss"], loss_fp64=loss64, rel_theta=rel(c5_gpu["theta"], gt),
           rel_path=rel(c5_gpu["path"], gp))
    assert abs(c5_gpu["loss"] - loss64) <= 1e-3 * loss64
    assert rel(c5_gpu["theta"], gt) <= 1e-3, rel(c5_gpu["theta"], gt)
    assert rel(c5_gpu["path"], gp) <= 1e-3, rel(c5_gpu["path"], gp)


def test_c5_gradient_matches_fp64_central_differences(c5_fp64, c5_gpu):
    """64 random directions in (log-compliance, capsule path); central differences of the FP64
    oracle's loss with step 1e-4 against the GPU gradient's directional derivatives."""
    c5 = c5_fp64.c5
    rng = np.random.default_rng(64)
    theta, path = c5.theta_initial.astype(np.float64), c5.path.astype(np.float64)
    eps, fd, an = 1e-4, [], []
    for _ in range(64):
        dth = rng.standard_normal(theta.shape)
        dpa = rng.standard_normal(path.shape) * 0.01
        up = c5_fp64.loss(theta + eps * dth, path + eps * dpa)
        dn = c5_fp64.loss(theta - eps * dth, path - eps * dpa)
        fd.append((up - dn) / (2 * eps))
        an.append(float((c5_gpu["theta"] * dth).sum() + (c5_gpu["path"] * dpa).sum()))
    record("c5_fp64_central_differences", directions=64, step=eps, rel=rel(an, fd))
    assert rel(an, fd) <= 1e-3, (rel(an, fd), an[:4], fd[:4])
