"""The CPU oracle against the reference's own outputs (tests/golden, written by
tests/golden/make_golden.py from the reference compiled from source).

These pin the oracle; the GPU tests then compare the CUDA path with the
oracle and with the same fixtures."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden


def scene_from(g):
    keys = ("extrinsics", "intrinsics", "points", "observations", "camera_index", "intrinsic_index",
            "point_index", "camera_constant", "intrinsic_constant")
    sc = {k: g[k] for k in keys}
    k = {0: 1, 1: 6, 2: 8}[int(g["model"])]
    sc["model"] = int(g["model"])
    sc["extrinsics"] = sc["extrinsics"].reshape(-1, 6)
    sc["intrinsics"] = sc["intrinsics"].reshape(-1, k)
    sc["points"] = sc["points"].reshape(-1, 3)
    sc["observations"] = sc["observations"].reshape(-1, 2)
    sc["intrinsic_fixed_mask"] = int(g["intrinsic_fixed_mask"])
    sc["extrinsic_fixed_mask"] = int(g["extrinsic_fixed_mask"])
    return sc


# ceres SPARSE_SCHUR solves (ba_iterative_* are ceres ITERATIVE_SCHUR runs and
# ba_illconditioned a tight-tolerance run, compared separately)
BA_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "ba_*.npz"))
                  if not os.path.basename(p).startswith(("ba_iterative", "ba_illconditioned")))
EVAL_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "eval_*.npz")))


def ba_options(abi, g):
    return abi.default_options(max_num_iterations=int(g["max_num_iterations"]), loss_type=int(g["loss"]),
                               loss_scale=float(g["loss_scale"]))


@pytest.mark.parametrize("case", BA_CASES)
def test_oracle_ba_matches_ceres(case, abi, oracle_mod):
    g = load_golden(case)
    sc = scene_from(g)
    st, s, prm, costs = oracle_mod.ba_solve(sc, ba_options(abi, g))
    assert st == 0 and s["usable"] == int(g["ref_usable"][0])
    ref_final = g["ref_final_cost"][0]
    assert abs(s["initial_cost"] - g["ref_initial_cost"][0]) <= 1e-12 * g["ref_initial_cost"][0]
    assert s["termination_type"] == int(g["ref_termination_type"][0])
    ref_costs = g["ref_iteration_cost"]
    if "percam" in case:
        # gauge-free scenes run to convergence: final-cost parity (1e-6 relative)
        assert abs(s["final_cost"] - ref_final) <= 1e-6 * ref_final
        assert abs(len(costs) - len(ref_costs)) <= 2
        n = min(len(costs), len(ref_costs), 10)
        np.testing.assert_allclose(costs[:n], ref_costs[:n], rtol=1e-8)
    else:
        # well-conditioned scenes: the same trajectory, iteration by iteration
        assert abs(s["final_cost"] - ref_final) <= 1e-9 * ref_final
        assert len(costs) == len(ref_costs), "same number of LM iterations as ceres"
        np.testing.assert_allclose(costs, ref_costs, rtol=1e-9)
        assert s["num_successful_steps"] == int(g["ref_num_successful_steps"][0])
        np.testing.assert_allclose(prm["points"].ravel(), g["ref_points"], rtol=0, atol=1e-7)
        np.testing.assert_allclose(prm["extrinsics"].ravel(), g["ref_extrinsics"], rtol=0, atol=1e-7)


def dense_jacobian(ev, sc, k):
    no = len(sc["observations"])
    nc, ni, npt = len(sc["extrinsics"]), len(sc["intrinsics"]), len(sc["points"])
    J = np.zeros((2 * no, 6 * nc + k * ni + 3 * npt))
    for o in range(no):
        c, i, p = sc["camera_index"][o], sc["intrinsic_index"][o], sc["point_index"][o]
        J[2 * o:2 * o + 2, 6 * c:6 * c + 6] = ev["jac_extrinsic"][o]
        J[2 * o:2 * o + 2, 6 * nc + k * i:6 * nc + k * i + k] = ev["jac_intrinsic"][o]
        J[2 * o:2 * o + 2, 6 * nc + k * ni + 3 * p:6 * nc + k * ni + 3 * p + 3] = ev["jac_point"][o]
    return J


def corrected(res, loss, a):
    s = (res ** 2).sum(1)
    scale = np.ones_like(s)
    if loss == 1:
        m = s > a * a
        scale[m] = np.sqrt(a / np.sqrt(s[m]))
    return res * scale[:, None]


@pytest.mark.parametrize("case", EVAL_CASES)
def test_oracle_jacobian_matches_ceres_autodiff(case, oracle_mod):
    g = load_golden(case)
    sc = scene_from(g)
    k = {0: 1, 1: 6, 2: 8}[sc["model"]]
    ev = oracle_mod.ba_evaluate(sc, int(g["loss"]), float(g["loss_scale"]))
    assert abs(ev["cost"] - g["ref_cost"][0]) <= 1e-12 * g["ref_cost"][0]
    np.testing.assert_allclose(corrected(ev["residuals"], int(g["loss"]), float(g["loss_scale"])).ravel(),
                               g["ref_residuals"], rtol=1e-12, atol=1e-9)
    J = dense_jacobian(ev, sc, k)
    Jr = g["ref_jacobian"].reshape(int(g["ref_jac_rows"][0]), int(g["ref_jac_cols"][0]))
    np.testing.assert_allclose(J, Jr, rtol=1e-10, atol=1e-9 * np.abs(Jr).max())
    np.testing.assert_allclose(ev["gradient"], g["ref_gradient"], rtol=1e-9, atol=1e-9 * np.abs(g["ref_gradient"]).max())


def same_up_to_sign(a, b, tol):
    a = a.reshape(-1, a.shape[-1])
    b = b.reshape(-1, b.shape[-1])
    s = np.sign((a * b).sum(1, keepdims=True))
    return np.abs(a * s - b).max() <= tol


@pytest.mark.parametrize("case", ["tri_ring_2x12.npz", "tri_ring_5x6.npz", "tri_noisy.npz"])
def test_oracle_triangulation_matches_reference(case, oracle_mod):
    g = load_golden(case)
    P = g["P"].reshape(-1, 12)
    off = g["track_offsets"].astype(np.int64)
    cam = g["camera_index"].astype(np.uint32)
    xy = g["xy"].reshape(-1, 2)
    nt = len(off) - 1
    first = off[:-1]
    Xh, Xe = oracle_mod.tri_dlt2(P[cam[first]], P[cam[first + 1]], xy[first], xy[first + 1])
    assert same_up_to_sign(Xh, g["dlt_h"].reshape(nt, 4), 1e-9)
    np.testing.assert_allclose(Xe, g["dlt_e"].reshape(nt, 3), rtol=1e-9, atol=1e-9)
    Xn, _ = oracle_mod.tri_nview(0, P, off, cam, xy)
    assert same_up_to_sign(Xn, g["nview_h"].reshape(nt, 4), 1e-9)
    Xa, _ = oracle_mod.tri_nview(1, P, off, cam, xy)
    assert same_up_to_sign(Xa, g["algebraic_h"].reshape(nt, 4), 1e-9)
    Xi, err = oracle_mod.tri_nview(2, P, off, cam, xy)
    np.testing.assert_allclose(Xi, g["iterative_e"].reshape(nt, 3), rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(err, g["iterative_error"], rtol=1e-6, atol=1e-9)


def test_reference_unit_test_assertions_hold_for_oracle(oracle_mod):
    """The reference's own triangulation assertions on its own scenes
    (triangulation_unittest.cpp:21 and triangulation_nview_unittest.cpp:32,62,86,91)."""
    g = load_golden("tri_ring_2x12.npz")
    P = g["P"].reshape(-1, 3, 4)
    xy = g["xy"].reshape(-1, 2)
    Xgt = g["X_gt"].reshape(-1, 3)
    _, Xe = oracle_mod.tri_dlt2(P[0].reshape(1, 12).repeat(12, 0), P[1].reshape(1, 12).repeat(12, 0),
                                xy[0::2], xy[1::2])
    assert np.abs(Xe - Xgt).max() < 1e-8
    g = load_golden("tri_ring_5x6.npz")
    P = g["P"].reshape(-1, 3, 4)
    off = g["track_offsets"].astype(np.int64)
    cam = g["camera_index"].astype(np.uint32)
    xy = g["xy"].reshape(-1, 2)
    for method in (0, 1):
        X, _ = oracle_mod.tri_nview(method, P.reshape(-1, 12), off, cam, xy)
        h = np.einsum("vij,tj->tvi", P, X)
        rep = h[..., :2] / h[..., 2:3]
        assert np.abs(rep - xy.reshape(6, 5, 2)).max() < 1e-9
    X, err = oracle_mod.tri_nview(2, P.reshape(-1, 12), off, cam, xy)
    assert err.max() < 1e-9


def illconditioned_options(abi):
    """The options the ill-conditioned fixture was solved with: ceres to a
    tight function tolerance (1e-12), at most 100 iterations, Huber(4)."""
    return abi.default_options(max_num_iterations=100, function_tolerance=1e-12, loss_type=abi.LOSS_HUBER,
                               loss_scale=4.0)


def test_oracle_illconditioned_reaches_ceres_minimum(abi, oracle_mod):
    """Twin cameras 0.01 apart, 40% of the points seen by one twin pair only:
    the FP64 restatement reaches ceres's minimum (both stop on the iteration
    limit or the tolerance near it)."""
    g = load_golden("ba_illconditioned.npz")
    st, s, _, _ = oracle_mod.ba_solve(scene_from(g), illconditioned_options(abi))
    ref = float(g["ref_final_cost"][0])
    assert st == 0 and s["usable"]
    assert abs(s["initial_cost"] - g["ref_initial_cost"][0]) <= 1e-12 * g["ref_initial_cost"][0]
    assert abs(s["final_cost"] - ref) <= 1e-9 * ref, (s["final_cost"], ref)
