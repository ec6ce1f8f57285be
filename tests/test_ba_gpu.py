"""GPU bundle adjustment through the C ABI against the oracle and the
reference's golden outputs.  Tolerances:
  - Jacobian blocks / residuals / gradient vs ceres AutoDiff: 1e-9 relative
    to the block scale (FP64; summation order differs);
  - final cost of the plain FP64 path vs ceres / oracle: 1e-6 relative (the
    parity bar), 1e-9 for the well-conditioned ring scenes;
  - mixed precision reaches the FP64 final cost within 1e-6 relative."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from test_oracle_golden import BA_CASES, EVAL_CASES, ba_options, corrected, dense_jacobian, scene_from

pytestmark = pytest.mark.gpu


def project(handle, abi, sc, loss=0, a=1.0, with_jac=True):
    hp = abi.HostProblem(sc)
    p = hp.struct()
    no = p.num_observations
    k = abi.MODEL_K[hp.model]
    res = np.zeros((no, 2))
    cost = np.zeros(1)
    handle.check(handle.lib.gbba_project_forward(handle.h, C.byref(p), loss, a, res.ctypes.data, cost.ctypes.data),
                 "forward")
    out = {"cost": cost[0], "residuals": res}
    if with_jac:
        je = np.zeros((no, 2, 6))
        ji = np.zeros((no, 2, k))
        jp = np.zeros((no, 2, 3))
        g = np.zeros(6 * p.num_cameras + k * p.num_intrinsics + 3 * p.num_points)
        handle.check(handle.lib.gbba_project_backward(handle.h, C.byref(p), loss, a, je.ctypes.data, ji.ctypes.data,
                                                      jp.ctypes.data, g.ctypes.data), "backward")
        out.update(jac_extrinsic=je, jac_intrinsic=ji, jac_point=jp, gradient=g)
    return out


@pytest.mark.parametrize("case", EVAL_CASES)
def test_forward_backward_match_ceres_autodiff(case, handle, abi):
    g = load_golden(case)
    sc = scene_from(g)
    loss, a = int(g["loss"]), float(g["loss_scale"])
    ev = project(handle, abi, sc, loss, a)
    assert abs(ev["cost"] - g["ref_cost"][0]) <= 1e-11 * g["ref_cost"][0]
    np.testing.assert_allclose(corrected(ev["residuals"], loss, a).ravel(), g["ref_residuals"], rtol=1e-11, atol=1e-9)
    k = abi.MODEL_K[sc["model"]]
    J = dense_jacobian(ev, sc, k)
    Jr = g["ref_jacobian"].reshape(int(g["ref_jac_rows"][0]), int(g["ref_jac_cols"][0]))
    np.testing.assert_allclose(J, Jr, rtol=1e-9, atol=1e-9 * np.abs(Jr).max())
    np.testing.assert_allclose(ev["gradient"], g["ref_gradient"], rtol=1e-8,
                               atol=1e-9 * np.abs(g["ref_gradient"]).max())


@pytest.mark.parametrize("model", [0, 1, 2])
def test_jacobian_central_differences(model, handle, abi, scenes):
    if model == 0:
        sc = scenes.ring_scene(num_cameras=3, num_points=8, seed=51, model=0)
        sc["extrinsics"][2, :3] = [0.0, 2e-9, -1e-9]  # first-order rotation branch
    else:
        sc = scenes.medium_scene(num_cameras=3, num_points=8, seed=52 + model, model=model)
    ev = project(handle, abi, sc)
    k = abi.MODEL_K[model]
    J = dense_jacobian(ev, sc, k)
    base = {f: sc[f].copy() for f in ("extrinsics", "intrinsics", "points")}
    cols = []
    for f in ("extrinsics", "intrinsics", "points"):
        for idx in range(base[f].size):
            h = 1e-6 * max(1.0, abs(base[f].flat[idx]))
            plus = dict(sc)
            minus = dict(sc)
            plus[f] = base[f].copy()
            minus[f] = base[f].copy()
            plus[f].flat[idx] += h
            minus[f].flat[idx] -= h
            rp = project(handle, abi, plus, with_jac=False)["residuals"].ravel()
            rm = project(handle, abi, minus, with_jac=False)["residuals"].ravel()
            cols.append((rp - rm) / (2 * h))
    Jfd = np.stack(cols, 1)
    if model == 0:
        # in the first-order branch ceres differentiates R p = p + w x p, not the exact rotation
        Jfd[:, 6 * 2:6 * 2 + 3] = J[:, 6 * 2:6 * 2 + 3]
    np.testing.assert_allclose(J, Jfd, rtol=2e-5, atol=2e-5 * np.abs(J).max())


def solve(handle, abi, sc, opts):
    hp = abi.HostProblem(sc)
    s = handle.solve(hp, opts)
    return s, hp.params()


@pytest.mark.parametrize("case", BA_CASES)
def test_fp64_solve_matches_ceres_golden(case, handle, abi):
    g = load_golden(case)
    sc = scene_from(g)
    s, prm = solve(handle, abi, sc, ba_options(abi, g))
    ref = g["ref_final_cost"][0]
    assert s.usable == 1
    assert abs(s.initial_cost - g["ref_initial_cost"][0]) <= 1e-11 * g["ref_initial_cost"][0]
    tol = 1e-6 if "percam" in case else 1e-9
    assert abs(s.final_cost - ref) <= tol * ref, (s.final_cost, ref)
    assert s.termination_type == int(g["ref_termination_type"][0])
    if "percam" not in case:
        assert s.num_iterations == len(g["ref_iteration_cost"]) - 1
        np.testing.assert_allclose(prm["points"].ravel(), g["ref_points"], rtol=0, atol=1e-6)


def test_fp64_solve_matches_oracle_ring(handle, abi, scenes, oracle_mod):
    sc = scenes.ring_scene(num_points=2000, seed=1)
    opts = scenes.ba_options_for(sc, max_num_iterations=20)
    s, prm = solve(handle, abi, sc, opts)
    _, so, po, costs = oracle_mod.ba_solve(sc, opts)
    assert abs(s.final_cost - so["final_cost"]) <= 1e-9 * so["final_cost"]
    assert s.num_iterations == so["num_iterations"]
    np.testing.assert_allclose(prm["points"], po["points"], atol=1e-8)
    np.testing.assert_allclose(prm["extrinsics"], po["extrinsics"], atol=1e-9)


@pytest.mark.parametrize("model", [1, 2])
def test_mixed_precision_reaches_fp64_cost(model, handle, abi, scenes):
    sc = scenes.medium_scene(num_cameras=20, num_points=1500, seed=60 + model, model=model)
    s64, _ = solve(handle, abi, sc, scenes.ba_options_for(sc, max_num_iterations=100))
    s32, _ = solve(handle, abi, sc, scenes.ba_options_for(sc, max_num_iterations=100, precision=abi.PRECISION_MIXED))
    assert s64.usable and s32.usable
    assert s32.final_cost <= s64.final_cost * (1 + 1e-6), (s32.final_cost, s64.final_cost)


def test_device_memory_problem_matches_host(handle, abi, scenes):
    torch = pytest.importorskip("torch")
    sc = scenes.medium_scene(num_cameras=10, num_points=400, seed=71)
    opts = scenes.ba_options_for(sc, max_num_iterations=15)
    s_h, prm_h = solve(handle, abi, sc, opts)
    dp = abi.DeviceProblem(sc)
    s_d = handle.solve(dp, opts)
    torch.cuda.synchronize()
    assert abs(s_d.final_cost - s_h.final_cost) <= 1e-9 * s_h.final_cost
    np.testing.assert_allclose(dp.params()["points"], prm_h["points"], atol=1e-7)


def test_unsorted_observations_same_result(handle, abi, scenes):
    sc = scenes.medium_scene(num_cameras=10, num_points=400, seed=72)
    opts = scenes.ba_options_for(sc, max_num_iterations=10)
    s1, p1 = solve(handle, abi, sc, opts)
    perm = np.random.default_rng(0).permutation(len(sc["observations"]))
    sc2 = dict(sc)
    for f in ("observations", "camera_index", "intrinsic_index", "point_index"):
        sc2[f] = sc[f][perm]
    s2, p2 = solve(handle, abi, sc2, opts)
    # observations are regrouped by point; only the order inside a point changes the rounding
    assert abs(s1.final_cost - s2.final_cost) <= 1e-9 * s1.final_cost


def test_invalid_index_rejected(handle, abi, scenes):
    sc = scenes.ring_scene(num_cameras=4, num_points=20, seed=73)
    sc["camera_index"] = sc["camera_index"].copy()
    sc["camera_index"][5] = 99
    hp = abi.HostProblem(sc)
    p = hp.struct()
    s = abi.GbbaSummary()
    st = handle.lib.gbba_solve(handle.h, C.byref(p), C.byref(abi.default_options()), C.byref(s))
    assert st == abi.ERROR_INVALID_ARGUMENT
    before = hp.points.copy()
    assert np.array_equal(hp.points, before)


def test_nonfinite_observation_reports_numerical_failure(handle, abi, scenes):
    sc = scenes.ring_scene(num_cameras=4, num_points=20, seed=74)
    sc["observations"] = sc["observations"].copy()
    sc["observations"][3, 0] = np.nan
    hp = abi.HostProblem(sc)
    p = hp.struct()
    s = abi.GbbaSummary()
    st = handle.lib.gbba_solve(handle.h, C.byref(p), C.byref(abi.default_options()), C.byref(s))
    assert st == abi.ERROR_NUMERICAL and s.usable == 0


def test_empty_and_all_constant_cameras(handle, abi, scenes):
    sc = scenes.ring_scene(num_cameras=4, num_points=30, seed=75)
    sc["camera_constant"] = np.ones(4, np.uint8)  # only points move: S is empty
    s, prm = solve(handle, abi, sc, scenes.ba_options_for(sc, max_num_iterations=10))
    assert s.usable and s.final_cost < s.initial_cost and s.reduced_system_size == 0
    empty = {"model": 1, "extrinsics": np.zeros((1, 6)), "intrinsics": np.zeros((1, 6)), "points": np.zeros((0, 3)),
             "observations": np.zeros((0, 2)), "camera_index": np.zeros(0, np.uint32),
             "intrinsic_index": np.zeros(0, np.uint32), "point_index": np.zeros(0, np.uint32)}
    s, _ = solve(handle, abi, empty, abi.default_options())
    assert s.initial_cost == 0.0 and s.usable
