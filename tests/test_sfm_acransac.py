"""AC-RANSAC hypothesis scoring of robustResection (gbsfm_acransac_score).

Fixtures (tests/golden/sfm_acransac_*.npz) come from the reference's own
ACRANSAC run with its six-point DLT kernel (unknown K) and its P3P kernel
(known K): every model the run drew, and the reference's score of each
(ResectionSquaredResidualError, std::sort, bestNFA with its float logcombi
tables).  The C++ and numpy oracles are pinned to them; the GPU scores are
compared with them: inlier counts exact, thresholds e[k-1] within 1e-12
relative, NFA within 1e-6 absolute (the logcombi tables are float-rounded
from log10 sums, and a device log10 a bit away from the host one can move a
table entry by one float ulp), and the replayed model selection gives the
reference's final inliers, threshold and minimum NFA."""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import load_golden

CASES = ["sfm_acransac_6pt.npz", "sfm_acransac_p3p.npz"]
NFA_TOL = 1e-6


def fixture_args(g):
    return (g["ref_x2d_normalized"].reshape(-1, 2), g["x3d"], g["ref_models"].reshape(-1, 12),
            int(g["ref_sample_size"][0]), int(g["ref_max_models"][0]), float(g["ref_logalpha0"][0]))


@pytest.mark.parametrize("case", CASES)
def test_oracle_scores_match_reference(case, oracle_mod):
    g = load_golden(case)
    nfa, k, emax, order, _ = oracle_mod.acransac_score_cpp(*fixture_args(g))
    np.testing.assert_array_equal(k, g["ref_k"].astype(np.int32))
    np.testing.assert_array_equal(nfa, g["ref_nfa"])
    np.testing.assert_array_equal(emax, g["ref_error_max"])
    nfa2, k2, emax2, _ = oracle_mod.acransac_score(*fixture_args(g))
    np.testing.assert_array_equal(k2, g["ref_k"].astype(np.int64))
    np.testing.assert_allclose(nfa2, g["ref_nfa"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("case", CASES)
def test_oracle_replay_matches_reference_run(case, oracle_mod):
    g = load_golden(case)
    nfa, k, emax, order, _ = oracle_mod.acransac_score_cpp(*fixture_args(g))
    err, min_nfa, inl, _ = oracle_mod.acransac_replay(nfa, k, emax, order, g["ref_models_per_fit"],
                                                      float(g["ref_normalizer"][0]))
    np.testing.assert_array_equal(inl, g["ref_result_inliers"].astype(np.int64))
    assert min_nfa == float(g["ref_result_min_nfa"][0])
    assert abs(err - float(g["ref_result_error_max"][0])) <= 1e-12 * abs(err)


def gpu_score(handle, abi, x2d, x3d, models, sample_size, max_models, logalpha0, max_threshold=math.inf,
              device=None, with_order=True):
    prm = abi.GbsfmAcransacParams(sample_size, max_models, logalpha0, 1.0, max_threshold)
    x2d = np.ascontiguousarray(x2d, np.float64)
    x3d = np.ascontiguousarray(x3d, np.float64)
    models = np.ascontiguousarray(models, np.float64)
    n, h = len(x2d), len(models)
    outs = [np.zeros(h), np.zeros(h, np.int32), np.zeros(h), np.zeros((h, n), np.uint32) if with_order else None]
    if device is None:
        ins = [x2d, x3d, models]
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        memory = abi.MEMORY_HOST
    else:
        import torch
        ins = [torch.from_numpy(a).to(device) for a in (x2d, x3d, models)]
        outs = [None if a is None else torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(device)
                for a in outs]
        ptr = lambda a: None if a is None else a.data_ptr()  # noqa: E731
        memory = abi.MEMORY_DEVICE
    st = handle.lib.gbsfm_acransac_score(handle.h, C.byref(prm), n, ptr(ins[0]), ptr(ins[1]), h, ptr(ins[2]),
                                         ptr(outs[0]), ptr(outs[1]), ptr(outs[2]), ptr(outs[3]), memory)
    if device is not None:
        outs = [None if a is None else a.cpu().numpy() for a in outs]
        if outs[3] is not None:
            outs[3] = outs[3].view(np.uint32)
    return st, outs


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("device", [None, "cuda:0"])
def test_gpu_scores_match_reference(case, device, handle, abi, oracle_mod):
    g = load_golden(case)
    st, (nfa, k, emax, order) = gpu_score(handle, abi, *fixture_args(g), device=device)
    handle.check(st, "gbsfm_acransac_score")
    np.testing.assert_array_equal(k, g["ref_k"].astype(np.int32))
    np.testing.assert_allclose(nfa, g["ref_nfa"], rtol=0, atol=NFA_TOL)
    np.testing.assert_allclose(emax, g["ref_error_max"], rtol=1e-12, atol=0)
    err, min_nfa, inl, _ = oracle_mod.acransac_replay(nfa, k, emax, order, g["ref_models_per_fit"],
                                                      float(g["ref_normalizer"][0]))
    np.testing.assert_array_equal(inl, g["ref_result_inliers"].astype(np.int64))
    assert abs(min_nfa - float(g["ref_result_min_nfa"][0])) <= NFA_TOL
    assert abs(err - float(g["ref_result_error_max"][0])) <= 1e-12 * abs(err)


def perturbed_models(g, count, seed, scale=0.02):
    """Models around the reference's best: its recorded models with relative
    noise, so that inlier counts spread."""
    rng = np.random.default_rng(seed)
    base = g["ref_models"].reshape(-1, 12)
    pick = base[rng.integers(0, len(base), count)]
    return pick * (1 + scale * rng.normal(size=pick.shape))


@pytest.mark.gpu
def test_gpu_threshold_and_unscored_models(handle, abi, oracle_mod):
    """A finite max_threshold cuts the scan; a model whose every error is
    above it scores NFA +inf with k = sample_size."""
    g = load_golden("sfm_acransac_6pt.npz")
    x2d, x3d, models, s, mm, la = fixture_args(g)
    models = np.concatenate([models[:40], np.array([[0, 0, 0, 1e6, 0, 0, 0, 1e6, 0, 0, 0, 1.0]])])
    thr = 1e-4
    st, (nfa, k, emax, order) = gpu_score(handle, abi, x2d, x3d, models, s, mm, la, max_threshold=thr)
    handle.check(st, "gbsfm_acransac_score")
    rn, rk, re, _, _ = oracle_mod.acransac_score_cpp(x2d, x3d, models, s, mm, la, max_threshold=thr)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_allclose(nfa, rn, rtol=0, atol=NFA_TOL)
    assert nfa[-1] == math.inf and k[-1] == s and emax[-1] == math.inf


@pytest.mark.gpu
@pytest.mark.parametrize("n", [7, 1000, 8192, 8193, 20000])
def test_gpu_sizes_match_oracle(n, handle, abi, oracle_mod, scenes):
    """Sizes around the shared-memory limit (8,192 pairs) and above it (the
    per-CTA global slice); the sorted order's first k (the inliers) exact."""
    g = load_golden("sfm_acransac_6pt.npz")
    sc = scenes.resection_scene(num_points=n, seed=100 + n)
    xn = (sc["x2d"] - np.array([sc["width"], sc["height"]]) / 2) / max(sc["width"], sc["height"])
    models = perturbed_models(g, 64, n)
    s, mm, la = 6, 1, math.log10(math.pi)
    st, (nfa, k, emax, order) = gpu_score(handle, abi, xn, sc["x3d"], models, s, mm, la)
    handle.check(st, "gbsfm_acransac_score")
    rn, rk, re, ro, _ = oracle_mod.acransac_score_cpp(xn, sc["x3d"], models, s, mm, la)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_allclose(nfa, rn, rtol=0, atol=NFA_TOL)
    np.testing.assert_allclose(emax, re, rtol=1e-12, atol=0)
    for h in range(len(models)):
        np.testing.assert_array_equal(np.sort(order[h, :k[h]]), np.sort(ro[h, :rk[h]]))


@pytest.mark.gpu
def test_gpu_rejects_too_few_points(handle, abi):
    x2d = np.zeros((6, 2))
    x3d = np.zeros((6, 3))
    st, _ = gpu_score(handle, abi, x2d, x3d, np.zeros((1, 12)), 6, 1, math.log10(math.pi))
    assert st == abi.ERROR_INVALID_ARGUMENT
