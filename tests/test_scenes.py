"""Synthetic scene generators: determinism, sizes, and projection sanity."""
import numpy as np


def test_ring_scene_shapes_and_visibility(scenes):
    sc = scenes.ring_scene()
    assert sc["extrinsics"].shape == (16, 6) and sc["points"].shape == (2000, 3)
    assert len(sc["observations"]) == 32000  # every point in frame for every camera
    t = sc["truth"]
    pred, depth = scenes.project(sc["model"], t["intrinsics"][sc["intrinsic_index"]],
                                 t["extrinsics"][sc["camera_index"]], t["points"][sc["point_index"]])
    assert (depth > 0).all()
    assert np.abs(pred - sc["observations"]).std() < 1.0  # sigma 0.5 px noise


def test_seeded_determinism(scenes):
    a = scenes.medium_scene(num_cameras=20, num_points=300, seed=5)
    b = scenes.medium_scene(num_cameras=20, num_points=300, seed=5)
    for k in ("extrinsics", "points", "observations", "camera_index"):
        assert np.array_equal(a[k], b[k])


def test_medium_views_are_distinct_per_point(scenes):
    sc = scenes.medium_scene(num_cameras=50, num_points=2000, seed=3)
    key = sc["point_index"].astype(np.int64) * 1000 + sc["camera_index"]
    assert len(np.unique(key)) == len(key)
    counts = np.bincount(sc["point_index"])
    assert counts.min() >= 2 and abs(counts.mean() - 10) < 0.5


def test_track_scene_csr(scenes):
    tr = scenes.track_scene(num_cameras=30, num_tracks=1000, seed=2)
    off = tr["track_offsets"]
    L = np.diff(off)
    assert off[0] == 0 and off[-1] == len(tr["camera_index"]) and L.min() >= 2 and L.max() <= 30


def test_angle_axis_round_trip(scenes):
    rng = np.random.default_rng(0)
    w = rng.normal(size=(100, 3))
    w *= (rng.uniform(0.01, 3.0, 100) / np.linalg.norm(w, axis=1))[:, None]
    np.testing.assert_allclose(scenes.rotation_to_angle_axis(scenes.angle_axis_to_rotation(w)), w, atol=1e-9)
