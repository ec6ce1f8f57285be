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
from test_oracle_golden import (BA_CASES, EVAL_CASES, ba_options, corrected, dense_jacobian, illconditioned_options,
                                scene_from)

pytestmark = pytest.mark.gpu


def project(handle, abi, sc, loss=0, a=1.0, with_jac=True, mixed=False):
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
        fn = handle.lib.gbba_project_backward_mixed if mixed else handle.lib.gbba_project_backward
        handle.check(fn(handle.h, C.byref(p), loss, a, je.ctypes.data, ji.ctypes.data, jp.ctypes.data, g.ctypes.data),
                     "backward")
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


def test_backward_gradient_is_bitwise_repeatable(handle, abi, scenes):
    """The gradient's per-parameter sums are fixed-point integer sums (a pass
    for each entry's largest term, then the scaled terms), so repeated calls
    give the same gradient bit for bit, in both precisions."""
    sc = scenes.medium_scene(num_cameras=30, num_points=4000, seed=151)
    for mixed in (False, True):
        runs = [project(handle, abi, sc, abi.LOSS_HUBER, 4.0, mixed=mixed)["gradient"] for _ in range(3)]
        assert np.all(np.isfinite(runs[0]))
        for g in runs[1:]:
            np.testing.assert_array_equal(g, runs[0])


# FP32 Jacobian of the mixed path: each entry within 2e-5 of the largest
# entry of its block type (extrinsic / intrinsic / point), i.e. a few hundred
# FP32 ulps of the block scale, which covers the rounding of the FP32 adjoint
# (rotation, distortion polynomial, division by depth) at pixel-scale values.
FP32_JAC_TOL = 2e-5


def assert_blocks_close(J, Jr, sc, k, tol):
    nc, ni = len(sc["extrinsics"]), len(sc["intrinsics"])
    for lo, hi in ((0, 6 * nc), (6 * nc, 6 * nc + k * ni), (6 * nc + k * ni, J.shape[1])):
        ref = Jr[:, lo:hi]
        scale = max(np.abs(ref).max(), 1e-300)
        np.testing.assert_allclose(J[:, lo:hi], ref, rtol=0, atol=tol * scale)


@pytest.mark.parametrize("case", EVAL_CASES)
def test_fp32_jacobian_matches_ceres_autodiff(case, handle, abi):
    """The FP32 Jacobian the mixed solve uses (gbba_project_backward_mixed)
    against ceres AutoDiff through Problem::Evaluate on the reference functors
    (autodiff_cost_function.h:202-211, problem.h:392-468)."""
    g = load_golden(case)
    sc = scene_from(g)
    loss, a = int(g["loss"]), float(g["loss_scale"])
    ev = project(handle, abi, sc, loss, a, mixed=True)
    k = abi.MODEL_K[sc["model"]]
    J = dense_jacobian(ev, sc, k)
    Jr = g["ref_jacobian"].reshape(int(g["ref_jac_rows"][0]), int(g["ref_jac_cols"][0]))
    assert_blocks_close(J, Jr, sc, k, FP32_JAC_TOL)
    # gradient J^T r (FP32 J, FP64 r): relative to the largest gradient entry
    np.testing.assert_allclose(ev["gradient"], g["ref_gradient"], rtol=0,
                               atol=FP32_JAC_TOL * np.abs(g["ref_gradient"]).max() * 10)


@pytest.mark.parametrize("model", [0, 1, 2])
def test_fp32_jacobian_central_differences(model, handle, abi, scenes):
    """The FP32 Jacobian against central differences of the FP64 residual on
    the medium workload's distributions (per-camera K3 and Brown-T2)."""
    if model == 0:
        sc = scenes.ring_scene(num_cameras=4, num_points=12, seed=57, model=0)
    else:
        sc = scenes.medium_scene(num_cameras=4, num_points=12, seed=57 + model, model=model)
    ev = project(handle, abi, sc, mixed=True)
    k = abi.MODEL_K[model]
    J = dense_jacobian(ev, sc, k)
    Jfd = central_differences(handle, abi, sc)
    assert_blocks_close(J, Jfd, sc, k, FP32_JAC_TOL)


def central_differences(handle, abi, sc):
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
    return np.stack(cols, 1)


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


def test_atomic_free_schur_matches_atomic_path(handle, abi, scenes):
    """The camera-pair (segmented, atomic-free) Schur build and the point-major
    atomic build give the same solve (FP64, well-posed scene)."""
    sc = scenes.medium_scene(num_cameras=25, num_points=1500, seed=101)
    sc["camera_constant"][1] = 1
    opts = scenes.ba_options_for(sc, max_num_iterations=15)
    s_pair, p_pair = solve(handle, abi, sc, opts)
    opts.schur_build = abi.SCHUR_BUILD_POINT_ATOMIC
    s_atom, p_atom = solve(handle, abi, sc, opts)
    assert s_pair.num_iterations == s_atom.num_iterations
    assert abs(s_pair.final_cost - s_atom.final_cost) <= 1e-10 * s_atom.final_cost
    np.testing.assert_allclose(p_pair["points"], p_atom["points"], atol=1e-8)


def test_autotune_keeps_the_fastest_work_item_size(gb, abi, scenes):
    """gbba_autotune times the Schur phase for each pair work-item size, keeps
    the fastest in the handle and leaves the problem's parameters unchanged;
    a solve with the tuned size reaches the default size's final cost."""
    sc = scenes.medium_scene(num_cameras=40, num_points=3000, seed=131)
    sc["camera_constant"][1] = 1
    opts = scenes.ba_options_for(sc, max_num_iterations=15)
    h = gb.Handle(0)  # its own handle: the tuned size stays with it
    try:
        s_ref, _ = solve(h, abi, sc, opts)
        hp = abi.HostProblem(sc)
        before = {k: v.copy() for k, v in hp.params().items()}
        tun = abi.GbbaTuning()
        p = hp.struct()
        st = h.lib.gbba_autotune(h.h, C.byref(p), C.byref(opts), 2, C.byref(tun))
        assert st == abi.SUCCESS
        assert tun.num_candidates == 3 and list(tun.candidates[:3]) == [32, 64, 128]
        times = list(tun.schur_time_s[:3])
        assert all(t > 0 for t in times)
        assert tun.pair_chunk == tun.candidates[times.index(min(times))]
        assert tun.factor_tensor == -1 and tun.camera_warps == 0  # FP64 dense: nothing else to tune
        for k, v in hp.params().items():
            np.testing.assert_array_equal(v, before[k])
        s_tuned = h.solve(hp, opts)
        assert s_tuned.usable
        assert abs(s_tuned.final_cost - s_ref.final_cost) <= 1e-9 * s_ref.final_cost
    finally:
        h.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("solver", ["dense", "pcg"])
def test_solves_are_bitwise_repeatable(handle, abi, scenes, solver, precision):
    """Every reduction of the camera-pair path has a fixed order (the first
    linearisation's column norms and gradient are fixed-point sums, the Schur
    blocks have one writer, the PCG sums are fixed-order partials), so
    repeated solves give the same parameters, costs and iteration counts bit
    for bit."""
    sc = scenes.medium_scene(num_cameras=40, num_points=3000, seed=141)
    sc["camera_constant"][1] = 1
    opts = scenes.ba_options_for(sc, max_num_iterations=12,
                                 precision=abi.PRECISION_MIXED if precision == "mixed" else abi.PRECISION_FP64)
    if solver == "pcg":
        opts.linear_solver = abi.SOLVER_ITERATIVE_SCHUR
    runs = [solve(handle, abi, sc, opts) for _ in range(3)]
    s0, p0 = runs[0]
    assert s0.usable
    for s1, p1 in runs[1:]:
        assert s1.final_cost == s0.final_cost and s1.num_iterations == s0.num_iterations
        for k in ("extrinsics", "intrinsics", "points"):
            np.testing.assert_array_equal(p1[k], p0[k])


@pytest.mark.parametrize("path", ["dense_mixed", "pcg_mixed"])
def test_autotune_factor_engine_and_camera_warps(gb, abi, scenes, path):
    """In mixed precision the autotuner also times the dense factorisation's
    trailing-update engine (tensor cores or FP32 pipes) or, on the PCG path,
    the warps per camera of the camera-side kernels, keeps the faster, and the
    tuned handle's solve reaches the untuned one's final cost within 1e-6."""
    sc = scenes.medium_scene(num_cameras=40, num_points=3000, seed=132)
    sc["camera_constant"][1] = 1
    opts = scenes.ba_options_for(sc, max_num_iterations=15, precision=abi.PRECISION_MIXED)
    if path == "pcg_mixed":
        opts.linear_solver = abi.SOLVER_ITERATIVE_SCHUR
    h = gb.Handle(0)
    try:
        s_ref, _ = solve(h, abi, sc, opts)
        hp = abi.HostProblem(sc)
        tun = abi.GbbaTuning()
        p = hp.struct()
        assert h.lib.gbba_autotune(h.h, C.byref(p), C.byref(opts), 2, C.byref(tun)) == abi.SUCCESS
        if path == "dense_mixed":
            ft = list(tun.factor_time_s)
            assert all(t > 0 for t in ft) and tun.factor_tensor == (1 if ft[1] <= ft[0] else 0)
            assert tun.camera_warps == 0
        else:
            pt = list(tun.pcg_time_s)
            assert all(t > 0 for t in pt) and tun.camera_warps == (2, 4, 8)[pt.index(min(pt))]
            assert tun.factor_tensor == -1
            assert tun.num_candidates == 0  # no camera-pair products on the iterative path
        s_tuned = h.solve(hp, opts)
        assert s_tuned.usable
        assert abs(s_tuned.final_cost - s_ref.final_cost) <= 1e-6 * s_ref.final_cost
    finally:
        h.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_cuda_graph_replay_matches_eager_launches(precision, handle, abi, scenes):
    sc = scenes.medium_scene(num_cameras=20, num_points=1000, seed=102)
    sc["camera_constant"][1] = 1
    a, pa = solve(handle, abi, sc, scenes.ba_options_for(sc, max_num_iterations=8, precision=precision,
                                                         use_cuda_graphs=1))
    b, pb = solve(handle, abi, sc, scenes.ba_options_for(sc, max_num_iterations=8, precision=precision,
                                                         use_cuda_graphs=0))
    # the column-norm reduction of the linearisation uses FP64 atomics, so two
    # runs agree to rounding, not bit for bit
    assert a.num_iterations == b.num_iterations
    assert abs(a.final_cost - b.final_cost) <= 1e-12 * b.final_cost
    np.testing.assert_allclose(pa["points"], pb["points"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("precision", [0, 1])
def test_iterative_schur_reaches_dense_minimum(precision, handle, abi, scenes):
    """Block-Jacobi PCG on the implicit Schur complement (the large-problem
    path) converges to the same minimum as the dense Cholesky."""
    sc = scenes.medium_scene(num_cameras=30, num_points=3000, seed=103)
    sc["camera_constant"][1] = 1
    kw = dict(max_num_iterations=200, function_tolerance=1e-12, precision=precision)
    d, _ = solve(handle, abi, sc, scenes.ba_options_for(sc, linear_solver=abi.SOLVER_DENSE_SCHUR, **kw))
    i, _ = solve(handle, abi, sc, scenes.ba_options_for(sc, linear_solver=abi.SOLVER_ITERATIVE_SCHUR, **kw))
    assert i.usable and i.linear_solver_iterations > 0
    assert abs(i.final_cost - d.final_cost) <= 1e-7 * d.final_cost, (i.final_cost, d.final_cost)


def test_iterative_schur_matches_ceres_iterative_schur(handle, abi):
    """Block-Jacobi PCG against ceres ITERATIVE_SCHUR with SCHUR_JACOBI
    (iterative_schur_complement_solver.cc:65-182, conjugate_gradients_solver.cc)
    on the same scene with the same forcing sequence (eta = 0.1) and stopping
    rule.  Intrinsics are held, so both preconditioners are the inverse 6x6
    camera blocks of S.  The truncated CG steps of two implementations differ
    in rounding, so the trajectories agree closely but not bit for bit: the
    first LM step's cost to 1e-6, the cost after 60 iterations to 1e-7."""
    g = load_golden("ba_iterative_k3.npz")
    sc = scene_from(g)
    o = ba_options(abi, g)
    o.linear_solver = abi.SOLVER_ITERATIVE_SCHUR
    o.function_tolerance = float(g["function_tolerance"])
    s, _ = solve(handle, abi, sc, o)
    ref = g["ref_iteration_cost"]
    assert s.usable and s.linear_solver_iterations > 0
    assert abs(s.initial_cost - ref[0]) <= 1e-11 * ref[0]
    o1 = ba_options(abi, g)
    o1.linear_solver = abi.SOLVER_ITERATIVE_SCHUR
    o1.max_num_iterations = 1
    s1, _ = solve(handle, abi, sc, o1)
    assert abs(s1.final_cost - ref[1]) <= 1e-6 * ref[1], (s1.final_cost, ref[1])
    assert abs(s.final_cost - g["ref_final_cost"][0]) <= 1e-7 * g["ref_final_cost"][0], \
        (s.final_cost, g["ref_final_cost"][0])
    # the CG work per LM step is of the same size as ceres's
    ref_cg = g["ref_iteration_linear_solver_iterations"].sum()
    assert 0.5 * ref_cg <= s.linear_solver_iterations <= 2.0 * ref_cg, (s.linear_solver_iterations, ref_cg)


WINDOW_CASES = ["ba_window_5.npz", "ba_window_20.npz", "ba_window_40.npz"]


def test_batched_windows_match_ceres(handle, abi):
    """Local-BA windows of the batched workload (Brown-T2, 5/20/40 cameras)
    in one gbba_solve_batched launch against ceres SPARSE_SCHUR on each: the
    FP64 kernel follows ceres's LM iteration by iteration (same iteration
    count, final cost to 1e-8 -- its FP64 reductions are atomic, so the
    rounding order varies), and the mixed kernel reaches ceres's final cost
    within 1e-6 (run with function tolerance 1e-8)."""
    gs = [load_golden(c) for c in WINDOW_CASES]
    scs = [scene_from(g) for g in gs]
    o64 = ba_options(abi, gs[0])
    st, sums, prms = batched_solve(handle, abi, scs, o64)
    assert st == abi.SUCCESS
    for g, s, prm in zip(gs, sums, prms):
        ref = g["ref_final_cost"][0]
        assert s.usable and abs(s.initial_cost - g["ref_initial_cost"][0]) <= 1e-11 * g["ref_initial_cost"][0]
        assert s.num_iterations == len(g["ref_iteration_cost"]) - 1
        assert abs(s.final_cost - ref) <= 1e-8 * ref, (s.final_cost, ref)
        np.testing.assert_allclose(prm["points"].ravel(), g["ref_points"], rtol=0, atol=1e-5)
    o32 = ba_options(abi, gs[0])
    o32.precision = abi.PRECISION_MIXED
    o32.function_tolerance = 1e-8
    o32.max_num_iterations = 200
    st, sums, _ = batched_solve(handle, abi, scs, o32)
    assert st == abi.SUCCESS
    for g, s in zip(gs, sums):
        ref = g["ref_final_cost"][0]
        assert s.usable and s.final_cost <= ref * (1 + 1e-6), (s.final_cost, ref)


def batched_solve(handle, abi, scenes_list, opts):
    hps = [abi.HostProblem(p) for p in scenes_list]
    n = len(hps)
    structs = (abi.GbbaProblem * n)(*[hp.struct() for hp in hps])
    sums = (abi.GbbaSummary * n)()
    st = handle.lib.gbba_solve_batched(handle.h, structs, n, C.byref(opts), sums)
    return st, list(sums), [hp.params() for hp in hps]


def local_problems(scenes, count, seed, cams=(5, 16), points=(200, 600)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        p = scenes.local_problem(rng, int(rng.integers(cams[0], cams[1] + 1)), int(rng.integers(points[0], points[1] + 1)))
        p["camera_constant"][1] = 1  # isolate the minimum (see the golden fixtures)
        out.append(p)
    return out


def test_batched_fp64_matches_individual_solves(handle, abi, scenes):
    """One launch, one CTA per problem: each window follows the same LM as
    gbba_solve and reaches the same final cost."""
    probs = local_problems(scenes, 12, seed=111)
    opts = abi.default_options(max_num_iterations=50)
    st, bs, bp = batched_solve(handle, abi, probs, opts)
    assert st == abi.SUCCESS
    for p, s, prm in zip(probs, bs, bp):
        si, pi = solve(handle, abi, p, opts)
        assert s.usable and si.usable
        assert abs(s.final_cost - si.final_cost) <= 1e-6 * si.final_cost, (s.final_cost, si.final_cost)
        assert abs(s.initial_cost - si.initial_cost) <= 1e-12 * si.initial_cost
        np.testing.assert_allclose(prm["points"], pi["points"], atol=1e-4)


def test_batched_fp64_large_windows_match_individual_solves(handle, abi, scenes):
    """FP64 windows of 31-40 cameras (reduced systems of 182-236 unknowns,
    above what an FP64 S in shared memory could hold) keep S in global memory
    and reach the same final cost as gbba_solve."""
    probs = local_problems(scenes, 6, seed=114, cams=(31, 40), points=(400, 900))
    opts = abi.default_options(max_num_iterations=50)
    st, bs, _ = batched_solve(handle, abi, probs, opts)
    assert st == abi.SUCCESS
    for p, s in zip(probs, bs):
        assert s.reduced_system_size > 176
        si, _ = solve(handle, abi, p, opts)
        assert s.usable and si.usable
        assert abs(s.final_cost - si.final_cost) <= 1e-6 * si.final_cost, (s.final_cost, si.final_cost)


def test_batched_mixed_reaches_fp64_cost(handle, abi, scenes):
    """Mixed-precision windows reach the FP64 minimum within 1e-6.  Some local
    windows have flat valleys in which ceres's default stopping rule
    (|dcost| <= 1e-6 cost) stops up to a few 1e-6 above the minimum, so the
    FP64 reference here is run with a tight function tolerance."""
    probs = local_problems(scenes, 16, seed=112, cams=(5, 40), points=(200, 600))
    o64 = abi.default_options(max_num_iterations=300, function_tolerance=1e-12)
    o32 = abi.default_options(max_num_iterations=100, precision=abi.PRECISION_MIXED)
    st, b32, _ = batched_solve(handle, abi, probs, o32)
    assert st == abi.SUCCESS
    for p, s in zip(probs, b32):
        si, _ = solve(handle, abi, p, o64)
        assert s.usable and s.final_cost <= si.final_cost * (1 + 1e-6), (s.final_cost, si.final_cost)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_solves_are_bitwise_repeatable(handle, abi, scenes, precision):
    """The Schur build's sums are fixed-point integer sums, so the order in
    which warps reach an entry cannot change them: repeated launches give the
    same parameters, costs and iteration counts bit for bit."""
    probs = local_problems(scenes, 24, seed=115, cams=(5, 40), points=(200, 1200))
    opts = abi.default_options(max_num_iterations=30)
    if precision == "mixed":
        opts = abi.default_options(max_num_iterations=30, precision=abi.PRECISION_MIXED)
    runs = [batched_solve(handle, abi, probs, opts) for _ in range(3)]
    for st, _, _ in runs:
        assert st == abi.SUCCESS
    _, s0, p0 = runs[0]
    for _, s1, p1 in runs[1:]:
        for a, b in zip(s0, s1):
            assert a.final_cost == b.final_cost and a.num_iterations == b.num_iterations
        for a, b in zip(p0, p1):
            for k in ("extrinsics", "intrinsics", "points"):
                np.testing.assert_array_equal(a[k], b[k])


def test_batched_multi_group_windows(handle, abi, scenes):
    """Windows with several intrinsic groups take the general Schur build
    (observation pairs for every column, no per-point intrinsic sums); a
    group shared by several cameras of one point tightens the fixed-point
    budget.  FP64 matches the individual solves, mixed reaches the FP64 cost,
    and both repeat bit for bit."""
    rng = np.random.default_rng(211)
    shapes = [(8, 300, 2), (12, 400, 3), (6, 250, 6), (10, 500, 4), (16, 600, 2)]
    probs = []
    for c, n, g in shapes:
        p = scenes.local_problem(rng, c, n, num_groups=g)
        p["camera_constant"][1] = 1
        probs.append(p)
    o64 = abi.default_options(max_num_iterations=100)
    st, bs, _ = batched_solve(handle, abi, probs, o64)
    assert st == abi.SUCCESS
    for p, s in zip(probs, bs):
        si, _ = solve(handle, abi, p, o64)
        assert s.usable and si.usable
        assert abs(s.final_cost - si.final_cost) <= 1e-6 * si.final_cost, (s.final_cost, si.final_cost)
    om = abi.default_options(max_num_iterations=200, precision=abi.PRECISION_MIXED)
    om.function_tolerance = 1e-8
    om.fp64_polish_iterations = 0
    runs = [batched_solve(handle, abi, probs, om) for _ in range(2)]
    for st_m, _, _ in runs:
        assert st_m == abi.SUCCESS
    for s64, a, b in zip(bs, runs[0][1], runs[1][1]):
        assert a.final_cost <= s64.final_cost * (1 + 1e-6), (a.final_cost, s64.final_cost)
        assert a.final_cost == b.final_cost and a.num_iterations == b.num_iterations
    for a, b in zip(runs[0][2], runs[1][2]):
        for k in ("extrinsics", "intrinsics", "points"):
            np.testing.assert_array_equal(a[k], b[k])


def test_batched_rejects_oversized_window(handle, abi, scenes):
    probs = local_problems(scenes, 2, seed=113)
    rng = np.random.default_rng(5)
    probs.append(scenes.local_problem(rng, 60, 300))  # 59*6 + 8 unknowns > 256
    st, _, _ = batched_solve(handle, abi, probs, abi.default_options(precision=abi.PRECISION_MIXED))
    assert st == abi.ERROR_TOO_LARGE


def test_illconditioned_fp64_matches_ceres(handle, abi):
    """The plain FP64 path on the ill-conditioned fixture (point blocks with
    condition ~1e6) reaches ceres's minimum."""
    g = load_golden("ba_illconditioned.npz")
    s, _ = solve(handle, abi, scene_from(g), illconditioned_options(abi))
    ref = float(g["ref_final_cost"][0])
    assert s.usable and abs(s.final_cost - ref) <= 1e-9 * ref, (s.final_cost, ref)


def _illcond_steps(handle, abi, g, iters, precision, flags=0):
    o = illconditioned_options(abi)
    o.max_num_iterations = iters
    o.precision = precision
    o.fp64_polish_iterations = 0
    o.mixed_flags = flags
    return solve(handle, abi, scene_from(g), o)


def test_fp64_point_inverse_reduces_step_error(handle, abi):
    """Three LM iterations from the ill-conditioned fixture's start in mixed
    precision, without and with the FP64 re-inversion of ill-conditioned
    point blocks (GBBA_MIXED_FP64_POINT_INVERSE), against the plain FP64 path.
    On the points seen by one twin pair only (condition ~1e6) the relative
    error of the parameters falls by more than a quarter (measured on GB300:
    1.0e-3 -> 4.8e-4); the other points and the cameras stay near the FP32
    level."""
    g = load_golden("ba_illconditioned.npz")
    sc = scene_from(g)
    pair = np.bincount(sc["point_index"].astype(np.int64), minlength=len(sc["points"])) == 2
    s64, p64 = _illcond_steps(handle, abi, g, 3, abi.PRECISION_FP64)
    step = np.linalg.norm(p64["points"][pair] - sc["points"][pair])
    err = {}
    for flags in (0, abi.MIXED_FP64_POINT_INVERSE):
        s, p = _illcond_steps(handle, abi, g, 3, abi.PRECISION_MIXED, flags)
        assert s.usable
        err[flags] = np.linalg.norm(p["points"][pair] - p64["points"][pair]) / step
        other = np.linalg.norm(p["points"][~pair] - p64["points"][~pair]) / np.linalg.norm(
            p64["points"][~pair] - sc["points"][~pair])
        assert other <= 1e-4, (flags, other)
    assert err[abi.MIXED_FP64_POINT_INVERSE] <= 0.75 * err[0], err


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_mixed_on_illconditioned_scene(handle, abi, flags):
    """The mixed path with each combination of its safeguards on the
    ill-conditioned fixture (100 iterations, no FP64 polish): usable, and its
    final cost within 2e-4 of ceres's (measured 9.5e-5 to 1.0e-4: the twin-pair
    points' depths are nearly free, and FP32 Jacobians slow their last
    digits)."""
    g = load_golden("ba_illconditioned.npz")
    s, _ = _illcond_steps(handle, abi, g, 100, abi.PRECISION_MIXED, flags)
    ref = float(g["ref_final_cost"][0])
    assert s.usable and (s.final_cost - ref) / ref <= 2e-4, s.final_cost
