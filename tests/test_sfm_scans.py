"""The engine-side scans around the bundle adjustment (include/gbsfm.h):
pair triangulation with its keep filter, bad-track rejection and residual
statistics.  The oracle's restatement is pinned to the reference's own
camera, DLT and histogram code (tests/golden/sfm_*.npz from ref_harness);
the GPU kernels are compared with the same fixtures.  Tolerances: points
and residuals 1e-9 relative (FP64), keep flags, counts and histogram bins
exact, float statistics exact (they are values of the sorted float array)
except the mean, within one float ulp."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

PAIRS = ["sfm_pair_resection.npz", "sfm_pair_initial.npz"]


def pair_inputs(g):
    return (g["cameras"].reshape(-1, 18), g["x1"].reshape(-1, 2), g["x2"].reshape(-1, 2), g["inlier"],
            float(g["max_residual"]), float(g["max_residual"]), float(g["min_angle"]))


@pytest.mark.parametrize("case", PAIRS)
def test_oracle_pair_matches_reference(case, oracle_mod):
    g = load_golden(case)
    X, res, keep = oracle_mod.sfm_triangulate_pair(*pair_inputs(g))
    np.testing.assert_allclose(X.ravel(), g["ref_X"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(res, g["ref_residual"], rtol=1e-9, atol=1e-12)
    np.testing.assert_array_equal(keep, g["ref_keep"].astype(np.uint8))


def test_oracle_tracks_match_reference(oracle_mod):
    g = load_golden("sfm_tracks.npz")
    args = (g["cameras"], g["points"], g["track_offsets"], g["camera_index"], g["xy"])
    ok, tk, nm, ntr = oracle_mod.sfm_reject_tracks(*args, precision=float(g["precision"]))
    np.testing.assert_array_equal(ok, g["ref_obs_keep"].astype(np.uint8))
    np.testing.assert_array_equal(tk, g["ref_track_keep"].astype(np.uint8))
    assert nm == int(g["ref_rejected_measurements"][0]) and ntr == int(g["ref_rejected_tracks"][0])
    st = oracle_mod.sfm_residual_histogram(*args)
    assert st["count"] == int(g["ref_hist_count"][0])
    for k in ("min", "max", "median"):
        assert st[k] == float(g[f"ref_hist_{k}"][0]), k
    assert abs(st["mean"] - float(g["ref_hist_mean"][0])) <= 1e-7 * abs(float(g["ref_hist_mean"][0]))
    np.testing.assert_array_equal(st["hist"], g["ref_hist_hist"].astype(np.int64))
    assert st["underflow"] == int(g["ref_hist_underflow"][0]) and st["overflow"] == int(g["ref_hist_overflow"][0])


def cameras_arg(cams):
    return np.ascontiguousarray(cams, np.float64).reshape(-1, 18)


@pytest.mark.gpu
@pytest.mark.parametrize("case", PAIRS)
def test_gpu_pair_matches_reference(case, handle, abi):
    g = load_golden(case)
    cams, x1, x2, inlier, th1, th2, ang = pair_inputs(g)
    cams = cameras_arg(cams)
    x1 = np.ascontiguousarray(x1)
    x2 = np.ascontiguousarray(x2)
    inl = np.ascontiguousarray(inlier, np.uint8)
    n = len(x1)
    X = np.zeros((n, 3))
    res = np.zeros(n)
    keep = np.zeros(n, np.uint8)
    kept = C.c_int64()
    handle.check(handle.lib.gbsfm_triangulate_pair(handle.h, cams[0].ctypes.data, cams[1].ctypes.data, n,
                                                   x1.ctypes.data, x2.ctypes.data, inl.ctypes.data, th1, th2, ang,
                                                   X.ctypes.data, res.ctypes.data, keep.ctypes.data,
                                                   C.byref(kept), abi.MEMORY_HOST), "gbsfm_triangulate_pair")
    np.testing.assert_allclose(X.ravel(), g["ref_X"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(res, g["ref_residual"], rtol=1e-9, atol=1e-12)
    np.testing.assert_array_equal(keep, g["ref_keep"].astype(np.uint8))
    assert kept.value == int(g["ref_keep"].sum())


@pytest.mark.gpu
def test_gpu_tracks_match_reference(handle, abi):
    g = load_golden("sfm_tracks.npz")
    cams = cameras_arg(g["cameras"])
    pts = np.ascontiguousarray(g["points"], np.float64)
    off = np.ascontiguousarray(g["track_offsets"], np.int64)
    cam = np.ascontiguousarray(g["camera_index"], np.uint32)
    xy = np.ascontiguousarray(g["xy"], np.float64)
    nt, no = len(off) - 1, len(cam)
    ok = np.zeros(no, np.uint8)
    tk = np.zeros(nt, np.uint8)
    nm, ntr = C.c_int64(), C.c_int64()
    handle.check(handle.lib.gbsfm_reject_tracks(handle.h, cams.ctypes.data, len(cams), pts.ctypes.data, nt,
                                                off.ctypes.data, cam.ctypes.data, xy.ctypes.data,
                                                float(g["precision"]), 3.0, ok.ctypes.data, tk.ctypes.data,
                                                C.byref(nm), C.byref(ntr), abi.MEMORY_HOST), "gbsfm_reject_tracks")
    np.testing.assert_array_equal(ok, g["ref_obs_keep"].astype(np.uint8))
    np.testing.assert_array_equal(tk, g["ref_track_keep"].astype(np.uint8))
    assert nm.value == int(g["ref_rejected_measurements"][0]) and ntr.value == int(g["ref_rejected_tracks"][0])
    st = abi.GbsfmResidualStats()
    handle.check(handle.lib.gbsfm_residual_histogram(handle.h, cams.ctypes.data, len(cams), pts.ctypes.data, nt,
                                                     off.ctypes.data, cam.ctypes.data, xy.ctypes.data, C.byref(st),
                                                     abi.MEMORY_HOST), "gbsfm_residual_histogram")
    assert st.count == int(g["ref_hist_count"][0])
    assert (st.min, st.max, st.median) == (float(g["ref_hist_min"][0]), float(g["ref_hist_max"][0]),
                                           float(g["ref_hist_median"][0]))
    assert abs(st.mean - float(g["ref_hist_mean"][0])) <= 1e-7 * abs(float(g["ref_hist_mean"][0]))
    assert list(st.hist) == [int(v) for v in g["ref_hist_hist"]]
    assert (st.underflow, st.overflow) == (int(g["ref_hist_underflow"][0]), int(g["ref_hist_overflow"][0]))


@pytest.mark.gpu
def test_gpu_tracks_order_inside_a_track_does_not_matter(handle, abi, oracle_mod):
    """The first ray of a track is the one of its lowest camera index, as in
    the reference's per-track map: shuffling the observations inside every
    track changes nothing; an out-of-range camera index is rejected."""
    g = load_golden("sfm_tracks.npz")
    off = g["track_offsets"].astype(np.int64)
    rng = np.random.default_rng(3)
    perm = np.concatenate([off[t] + rng.permutation(off[t + 1] - off[t]) for t in range(len(off) - 1)])
    cams = cameras_arg(g["cameras"])
    pts = np.ascontiguousarray(g["points"])
    cam = np.ascontiguousarray(g["camera_index"][perm], np.uint32)
    xy = np.ascontiguousarray(g["xy"][perm])
    ok = np.zeros(len(cam), np.uint8)
    nm, ntr = C.c_int64(), C.c_int64()
    handle.check(handle.lib.gbsfm_reject_tracks(handle.h, cams.ctypes.data, len(cams), pts.ctypes.data, len(off) - 1,
                                                off.ctypes.data, cam.ctypes.data, xy.ctypes.data, 4.0, 3.0,
                                                ok.ctypes.data, None, C.byref(nm), C.byref(ntr), abi.MEMORY_HOST),
                 "reject (shuffled)")
    np.testing.assert_array_equal(ok, g["ref_obs_keep"].astype(np.uint8)[perm])
    assert nm.value == int(g["ref_rejected_measurements"][0]) and ntr.value == int(g["ref_rejected_tracks"][0])
    cam[5] = len(cams) + 3
    st = handle.lib.gbsfm_reject_tracks(handle.h, cams.ctypes.data, len(cams), pts.ctypes.data, len(off) - 1,
                                        off.ctypes.data, cam.ctypes.data, xy.ctypes.data, 4.0, 3.0, None, None,
                                        None, None, abi.MEMORY_HOST)
    assert st == abi.ERROR_INVALID_ARGUMENT
