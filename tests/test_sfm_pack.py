"""Problem assembly and write-back of the incremental engine's bundle
adjustment (gbsfm_pack_ba / gbsfm_unpack_ba in include/gbsfm.h).

The oracle restatement is pinned to the reference harness (BundleAdjustment's
loops over its own std::map state with ceres's RotationMatrixToAngleAxis /
AngleAxisToRotationMatrix, tests/golden/sfm_pack.npz).  The GPU pack is
compared with the same fixture: indices, observations, the locked block and
the counts exactly; angle-axis values within 1e-14 (the device atan2 and the
host one may differ in the last bit); the written-back rotations within
1e-15.  At full size (5,000 images, 2M tracks, ~10M entries) the GPU pack is
compared with the oracle on every index and observation, and the
pack -> write-back round trip gives the original rotations back."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

ANGLE_TOL = 1e-14
ROT_TOL = 1e-15


def ref_split(g):
    nc = int(g["ref_num_cameras"][0])
    ng = len(g["group_keys"])
    p = g["ref_parameters"]
    return nc, p[:6 * nc].reshape(-1, 6), p[6 * nc:6 * nc + 6 * ng], p[6 * nc + 6 * ng:]


def test_oracle_pack_matches_reference(oracle_mod):
    g = load_golden("sfm_pack.npz")
    o = oracle_mod.sfm_pack(g)
    nc, ext, _, _ = ref_split(g)
    assert o["num_cameras"] == nc
    np.testing.assert_array_equal(o["extrinsics"], ext)
    np.testing.assert_array_equal(o["observations"].ravel(), g["ref_observations"])
    np.testing.assert_array_equal(o["camera_index"], g["ref_camera_index_extrinsic"].astype(np.uint32))
    np.testing.assert_array_equal(o["intrinsic_index"], g["ref_camera_index_intrinsic"].astype(np.uint32))
    np.testing.assert_array_equal(o["point_index"], g["ref_point_index"].astype(np.uint32))
    assert o["measurements"] == int(g["ref_measurements"][0])
    assert o["locked_camera"] == int(g["ref_locked"][0])


def test_oracle_unpack_matches_reference(oracle_mod):
    g = load_golden("sfm_pack.npz")
    o = oracle_mod.sfm_pack(g)
    u = oracle_mod.sfm_unpack(g["refined_extrinsics"], o["camera_image"], g["refined_intrinsics"],
                              g["intrinsic_group"], g["cameras"])
    np.testing.assert_allclose(u[o["camera_image"]], g["ref_unpacked"].reshape(-1, 18), rtol=0, atol=ROT_TOL)


def test_oracle_rotation_branches(oracle_mod):
    """Every branch of the conversion round-trips: the trace test, each
    largest-diagonal case, the zero rotation and the half turns."""
    rng = np.random.default_rng(3)
    cases = [np.zeros(3), np.array([1e-9, 0, 0]), np.array([np.pi, 0, 0]), np.array([0, np.pi, 0]),
             np.array([0, 0, np.pi]), np.array([0.6, -0.8, 0.0]) * (np.pi - 1e-6)] + list(rng.normal(0, 1, (20, 3)))
    for aa in cases:
        R = oracle_mod.angle_axis_to_rotation(aa)
        back = oracle_mod.angle_axis_to_rotation(oracle_mod.rotation_to_angle_axis(R))
        np.testing.assert_allclose(back, R, atol=1e-12)


def lock_state(scenes, first, rec_first=True):
    st = scenes.engine_state(num_images=12, num_points=40, seed=4)
    st["first_added"] = first
    st["reconstructed"] = st["reconstructed"].copy()
    st["reconstructed"][first] = 1 if rec_first else 0
    return st


def test_oracle_lock_modes(oracle_mod, scenes):
    st = lock_state(scenes, 6)
    ordinal = int(np.cumsum(st["reconstructed"] != 0)[6] - 1)
    ref = oracle_mod.sfm_pack(st, lock=0)
    assert ref["locked_camera"] == int(ref["camera_index"][ordinal])
    assert oracle_mod.sfm_pack(st, lock=1)["locked_camera"] == ordinal
    assert oracle_mod.sfm_pack(st, lock=2)["locked_camera"] == -1
    st = lock_state(scenes, 6, rec_first=False)
    # std::map::operator[] gives the missing image ordinal 0
    assert oracle_mod.sfm_pack(st, lock=0)["locked_camera"] == int(oracle_mod.sfm_pack(st)["camera_index"][0])
    assert oracle_mod.sfm_pack(st, lock=1)["locked_camera"] == -1


# ---------------------------------------------------------------- GPU


def gpu_pack(handle, abi, state, device=None, lock=0):
    ep = abi.EnginePack(state, device)
    st, o = ep.pack(handle.lib, handle.h, int(state["first_added"]), lock)
    return st, ep, o


def check_against(res, o, ext_tol=ANGLE_TOL):
    assert res["num_cameras"] == o["num_cameras"]
    np.testing.assert_allclose(res["extrinsics"], o["extrinsics"], rtol=0, atol=ext_tol)
    np.testing.assert_array_equal(res["camera_image"], o["camera_image"])
    np.testing.assert_array_equal(res["observations"], o["observations"])
    for k in ("camera_index", "intrinsic_index", "point_index"):
        np.testing.assert_array_equal(res[k], o[k], err_msg=k)
    assert res["measurements"] == o["measurements"]
    assert res["locked_camera"] == o["locked_camera"]


@pytest.mark.gpu
@pytest.mark.parametrize("device", [None, "cuda:0"])
def test_gpu_pack_matches_reference(handle, abi, oracle_mod, device):
    g = load_golden("sfm_pack.npz")
    st, ep, o = gpu_pack(handle, abi, g, device)
    handle.check(st, "gbsfm_pack_ba")
    res = ep.result(o)
    nc, ext, intr, pts = ref_split(g)
    assert res["num_cameras"] == nc and res["num_observations"] == len(g["ref_point_index"])
    np.testing.assert_allclose(res["extrinsics"], ext, rtol=0, atol=ANGLE_TOL)
    np.testing.assert_array_equal(res["intrinsics"], intr)
    np.testing.assert_array_equal(res["points"], pts)
    np.testing.assert_array_equal(res["observations"].ravel(), g["ref_observations"])
    np.testing.assert_array_equal(res["camera_index"], g["ref_camera_index_extrinsic"].astype(np.uint32))
    np.testing.assert_array_equal(res["intrinsic_index"], g["ref_camera_index_intrinsic"].astype(np.uint32))
    np.testing.assert_array_equal(res["point_index"], g["ref_point_index"].astype(np.uint32))
    assert res["measurements"] == int(g["ref_measurements"][0])
    assert res["locked_camera"] == int(g["ref_locked"][0])
    cc = np.zeros(nc, np.uint8)
    cc[res["locked_camera"]] = 1
    np.testing.assert_array_equal(res["camera_constant"], cc)


@pytest.mark.gpu
@pytest.mark.parametrize("device", [None, "cuda:0"])
def test_gpu_unpack_matches_reference(handle, abi, device):
    g = load_golden("sfm_pack.npz")
    st, ep, o = gpu_pack(handle, abi, g)
    handle.check(st, "gbsfm_pack_ba")
    cimg = ep.result(o)["camera_image"].copy()
    cams = np.ascontiguousarray(g["cameras"], np.float64).copy()
    arrs = [np.ascontiguousarray(g["refined_extrinsics"], np.float64), cimg,
            np.ascontiguousarray(g["refined_intrinsics"], np.float64),
            np.ascontiguousarray(g["intrinsic_group"], np.uint32), cams]
    memory = abi.MEMORY_HOST
    if device is not None:
        import torch
        arrs = [torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(device) for a in arrs]
        memory = abi.MEMORY_DEVICE
    ptr = [a.ctypes.data if device is None else a.data_ptr() for a in arrs]
    handle.check(handle.lib.gbsfm_unpack_ba(handle.h, len(cimg), ptr[0], ptr[1], ptr[2], len(g["group_keys"]), ptr[3],
                                            len(cams), ptr[4], memory), "gbsfm_unpack_ba")
    out = cams if device is None else arrs[4].cpu().numpy()
    np.testing.assert_allclose(out[cimg], g["ref_unpacked"].reshape(-1, 18), rtol=0, atol=ROT_TOL)
    untouched = np.setdiff1d(np.arange(len(cams)), cimg)
    np.testing.assert_array_equal(out[untouched], g["cameras"][untouched])


@pytest.mark.gpu
@pytest.mark.parametrize("lock", [0, 1, 2])
@pytest.mark.parametrize("rec_first", [True, False])
def test_gpu_lock_modes(handle, abi, oracle_mod, scenes, lock, rec_first):
    st = lock_state(scenes, 6, rec_first)
    s, ep, o = gpu_pack(handle, abi, st, lock=lock)
    handle.check(s, "gbsfm_pack_ba")
    check_against(ep.result(o), oracle_mod.sfm_pack(st, lock=lock))


@pytest.mark.gpu
def test_gpu_pack_edge_cases(handle, abi, oracle_mod, scenes):
    # no image reconstructed: no camera, no observation, no lock
    st = scenes.engine_state(num_images=10, num_points=30, seed=5)
    st["reconstructed"] = np.zeros(10, np.uint8)
    s, ep, o = gpu_pack(handle, abi, st)
    handle.check(s, "gbsfm_pack_ba")
    r = ep.result(o)
    assert r["num_cameras"] == 0 and r["num_observations"] == 0 and r["locked_camera"] == -1
    assert r["measurements"] == len(st["track_image"])
    # no engine image added yet
    st = scenes.engine_state(num_images=10, num_points=30, seed=5)
    st["first_added"] = -1
    s, ep, o = gpu_pack(handle, abi, st)
    handle.check(s, "gbsfm_pack_ba")
    check_against(ep.result(o), oracle_mod.sfm_pack(st))
    # empty tracks and a track list without entries
    st = scenes.engine_state(num_images=10, num_points=30, seed=5)
    off = st["track_offsets"].copy()
    off[5:] = off[5]
    st["track_offsets"] = off
    st["track_image"] = st["track_image"][:off[-1]]
    st["track_feature"] = st["track_feature"][:off[-1]]
    s, ep, o = gpu_pack(handle, abi, st)
    handle.check(s, "gbsfm_pack_ba")
    check_against(ep.result(o), oracle_mod.sfm_pack(st))
    # more than one tile of entries with most images dropped
    st = scenes.engine_state(num_images=60, num_points=3000, seed=6, reconstructed_frac=0.2)
    s, ep, o = gpu_pack(handle, abi, st)
    handle.check(s, "gbsfm_pack_ba")
    check_against(ep.result(o), oracle_mod.sfm_pack(st))


@pytest.mark.gpu
@pytest.mark.parametrize("fault", ["image", "feature", "offsets", "group", "first_added"])
def test_gpu_pack_rejects_invalid_state(handle, abi, scenes, fault):
    st = scenes.engine_state(num_images=10, num_points=30, seed=5)
    first = st["first_added"]
    if fault == "image":
        st["track_image"] = st["track_image"].copy()
        st["track_image"][7] = 10
    elif fault == "feature":
        st["track_feature"] = st["track_feature"].copy()
        im = st["track_image"][3]
        st["track_feature"][3] = st["feature_offsets"][im + 1] - st["feature_offsets"][im]
    elif fault == "offsets":
        st["track_offsets"] = st["track_offsets"].copy()
        st["track_offsets"][4] = st["track_offsets"][3] - 1
    elif fault == "group":
        st["intrinsic_group"] = st["intrinsic_group"].copy()
        st["intrinsic_group"][np.flatnonzero(st["reconstructed"])[0]] = 3
    else:
        first = 10
    ep = abi.EnginePack(st)
    s, _ = ep.pack(handle.lib, handle.h, first)
    assert s == abi.ERROR_INVALID_ARGUMENT
    # the handle stays usable
    s, o = abi.EnginePack(scenes.engine_state(num_images=10, num_points=30, seed=5)).pack(handle.lib, handle.h, 7)
    handle.check(s, "gbsfm_pack_ba")


@pytest.mark.gpu
def test_gpu_unpack_rejects_bad_ordinal(handle, abi):
    cams = np.zeros((4, 18))
    cams_before = cams.copy()
    ext = np.zeros((2, 6))
    cimg = np.array([1, 4], np.uint32)
    intr = np.ones((1, 6))
    grp = np.zeros(4, np.uint32)
    s = handle.lib.gbsfm_unpack_ba(handle.h, 2, ext.ctypes.data, cimg.ctypes.data, intr.ctypes.data, 1,
                                   grp.ctypes.data, 4, cams.ctypes.data, abi.MEMORY_HOST)
    assert s == abi.ERROR_INVALID_ARGUMENT
    np.testing.assert_array_equal(cams, cams_before)


@pytest.mark.gpu
def test_gpu_pack_feeds_the_solver(handle, abi, oracle_mod):
    """The packed problem is a GBBA_MODEL_RADIAL_K3 problem as it stands:
    its cost at the packed parameters equals the oracle's on the same arrays."""
    g = load_golden("sfm_pack.npz")
    s, ep, o = gpu_pack(handle, abi, g)
    handle.check(s, "gbsfm_pack_ba")
    r = ep.result(o)
    sc = {"model": abi.RADIAL_K3, "extrinsics": r["extrinsics"], "intrinsics": r["intrinsics"],
          "points": r["points"], "observations": r["observations"], "camera_index": r["camera_index"],
          "intrinsic_index": r["intrinsic_index"], "point_index": r["point_index"],
          "camera_constant": r["camera_constant"]}
    hp = abi.HostProblem(sc)
    p = hp.struct()
    cost = C.c_double()
    res = np.zeros(2 * r["num_observations"])
    handle.check(handle.lib.gbba_project_forward(handle.h, C.byref(p), abi.LOSS_SQUARED, 1.0, res.ctypes.data,
                                                 C.byref(cost)), "gbba_project_forward")
    want = oracle_mod.ba_evaluate(sc)["cost"]
    assert np.isfinite(cost.value) and abs(cost.value - want) <= 1e-9 * abs(want)


@pytest.mark.gpu
def test_gpu_pack_full_size(handle, abi, oracle_mod, scenes):
    """5,000 images (~4,000 reconstructed), 2M tracks, ~10M entries: every
    index and observation as the oracle's, and the write-back of the packed
    extrinsics gives the cameras' rotations back."""
    import torch
    st = scenes.engine_state_large()
    s, ep, o = gpu_pack(handle, abi, st, device="cuda:0")
    handle.check(s, "gbsfm_pack_ba")
    res = ep.result(o)
    check_against(res, oracle_mod.sfm_pack(st), ext_tol=1e-13)
    nc = res["num_cameras"]
    cams = ep.arrays["cameras"].clone()
    ext = ep.out["extrinsics"][:6 * nc].clone()
    ext[3::6] += 1.0  # a moved translation shows the write-back ran
    handle.check(handle.lib.gbsfm_unpack_ba(handle.h, nc, ext.data_ptr(), ep.out["camera_image"].data_ptr(),
                                            ep.arrays["group_intrinsics"].data_ptr(), ep.ng,
                                            ep.arrays["intrinsic_group"].data_ptr(), ep.ni, cams.data_ptr(),
                                            abi.MEMORY_DEVICE), "gbsfm_unpack_ba")
    back = cams.cpu().numpy().reshape(-1, 18)
    ci = res["camera_image"].astype(np.int64)
    orig = np.asarray(st["cameras"]).reshape(-1, 18)
    np.testing.assert_allclose(back[ci, :9], orig[ci, :9], atol=1e-13)
    np.testing.assert_array_equal(back[ci, 9], orig[ci, 9] + 1.0)
    del torch
