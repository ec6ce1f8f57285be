"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs oracle/_ref/ref_harness -- the reference's own code (its ceres
functors + vendored ceres 1.10 / CXSparse / Eigen, and libs/multiview
triangulation) compiled from the reference sources by `make -C oracle ref` --
on small seeded inputs and stores inputs and outputs as .npz files.  Needs the
reference sources, so it runs in the development container only; the
fixtures it writes are committed and travel with the tests.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py tri_long   # named groups only
"""
import importlib
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

abi = importlib.import_module("3dreconstruction_gb300.abi")
scenes = importlib.import_module("3dreconstruction_gb300.scenes")
OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, **arrays):
    np.savez_compressed(os.path.join(OUT, name), **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", name)


def tri_ring(tmp, nviews, npoints):
    """The scenes of the reference's triangulation unit tests
    (libs/multiview/src/triangulation_unittest.cpp:12,
    triangulation_nview_unittest.cpp:9) with the reference outputs."""
    r = oracle.ref_run("tri-ring", None, tmp, extra_args=(nviews, npoints))
    save(f"tri_ring_{nviews}x{npoints}.npz", **r)


def tri_noisy(tmp):
    tr = scenes.track_scene(num_cameras=24, num_tracks=300, seed=21, max_len=12)
    r = oracle.ref_run("tri", {"P": tr["P"], "track_offsets": tr["track_offsets"],
                               "camera_index": tr["camera_index"], "xy": tr["xy"]}, tmp)
    save("tri_noisy.npz", P=tr["P"], track_offsets=tr["track_offsets"], camera_index=tr["camera_index"],
         xy=tr["xy"], **r)


def scene_arrays(sc):
    keys = ("extrinsics", "intrinsics", "points", "observations", "camera_index", "intrinsic_index", "point_index")
    out = {k: sc[k] for k in keys}
    out["model"] = sc["model"]
    out["camera_constant"] = sc.get("camera_constant") if sc.get("camera_constant") is not None else np.zeros(len(sc["extrinsics"]), np.uint8)
    out["intrinsic_constant"] = sc.get("intrinsic_constant") if sc.get("intrinsic_constant") is not None else np.zeros(len(sc["intrinsics"]), np.uint8)
    out["intrinsic_fixed_mask"] = sc.get("intrinsic_fixed_mask", 0)
    out["extrinsic_fixed_mask"] = sc.get("extrinsic_fixed_mask", 0)
    return out


def ba_case(tmp, name, sc, layout=0, **opt):
    o = scenes.ba_options_for(sc, **opt)
    r = oracle.ref_run("ba", oracle.scene_to_kv(sc, o, layout=layout, linear_solver=0), tmp)
    save(f"ba_{name}.npz", layout=layout, loss=o.loss_type, loss_scale=o.loss_scale,
         max_num_iterations=o.max_num_iterations, **scene_arrays(sc),
         **{"ref_" + k: v for k, v in r.items()})


def eval_case(tmp, name, sc, loss=0, a=1.0):
    o = scenes.ba_options_for(sc, loss_type=loss, loss_scale=a)
    r = oracle.ref_run("eval", oracle.scene_to_kv(sc, o), tmp)
    save(f"eval_{name}.npz", loss=loss, loss_scale=a, **scene_arrays(sc), **{"ref_" + k: v for k, v in r.items()})


def unit_test_scene(tmp):
    """The reference's BA unit test (libs/sfm/src/bundle_adjustment_unittest.cpp:
    19-122): NRealisticCamerasRing(3,6), [R t f] blocks, observations centred by
    the principal point (500,500) and shifted by its integer-division "noise"
    rand()/RAND_MAX - 0.5 = -0.5, squared loss."""
    r = oracle.ref_run("tri-ring", None, tmp, extra_args=(3, 6))
    P = r["P"].reshape(3, 3, 4)
    R = r["R"].reshape(3, 3, 3)
    t = r["t"].reshape(3, 3)
    X = r["X_gt"].reshape(6, 3)
    xy = r["xy"].reshape(-1, 2)
    cam = r["camera_index"].astype(np.uint32)
    pt = np.repeat(np.arange(6), 3).astype(np.uint32)
    obs = xy - 500.0 - 0.5
    ext = np.concatenate([scenes.rotation_to_angle_axis(R), t], 1)
    sc = {"model": abi.PINHOLE_F, "extrinsics": ext, "intrinsics": np.full((3, 1), 1000.0), "points": X,
          "observations": obs, "camera_index": cam, "intrinsic_index": cam.copy(), "point_index": pt}
    return sc, P


def tri_tracks_f32(tmp):
    """Tracks of the batched-triangulation workload's distributions (200
    cameras on a sphere of radius 15, f in [800,1200], lengths 2-30, 1 px
    noise), with P and the pixels rounded to FP32 before the reference sees
    them, so that the FP32 path and the reference get identical inputs."""
    tr = scenes.track_scene(num_cameras=200, num_tracks=6000, seed=22)
    P = tr["P"].astype(np.float32).astype(np.float64)
    xy = tr["xy"].astype(np.float32).astype(np.float64)
    r = oracle.ref_run("tri", {"P": P, "track_offsets": tr["track_offsets"], "camera_index": tr["camera_index"],
                               "xy": xy}, tmp)
    save("tri_tracks_f32.npz", P=P.astype(np.float32), track_offsets=tr["track_offsets"].astype(np.uint32),
         camera_index=tr["camera_index"].astype(np.uint8), xy=xy.astype(np.float32), X_true=tr["X_true"], **r)


def tri_long(tmp):
    """Tracks of 33-150 views (beyond a 32-view warp), as the global engine's
    per-track loop can produce (sfm_global_engine.cpp:597-651)."""
    tr = scenes.track_scene(num_cameras=160, num_tracks=40, seed=23, min_len=33, max_len=150)
    r = oracle.ref_run("tri", {"P": tr["P"], "track_offsets": tr["track_offsets"],
                               "camera_index": tr["camera_index"], "xy": tr["xy"]}, tmp)
    save("tri_long.npz", P=tr["P"], track_offsets=tr["track_offsets"], camera_index=tr["camera_index"],
         xy=tr["xy"], **r)


def ba_iterative(tmp):
    """ceres ITERATIVE_SCHUR with the SCHUR_JACOBI preconditioner (the block
    diagonal of the reduced camera system, as the GPU PCG uses) on a per-camera
    K3 scene whose intrinsics are held, so that both preconditioners are the
    same 6x6 camera blocks; run to a tight function tolerance."""
    sc = scenes.medium_scene(num_cameras=24, num_points=1200, seed=38)
    sc["camera_constant"][1] = 1
    sc["intrinsic_constant"] = np.ones(len(sc["intrinsics"]), np.uint8)
    o = scenes.ba_options_for(sc, max_num_iterations=60, function_tolerance=1e-10)
    r = oracle.ref_run("ba", oracle.scene_to_kv(sc, o, linear_solver=2, preconditioner=1), tmp)
    save("ba_iterative_k3.npz", layout=0, loss=o.loss_type, loss_scale=o.loss_scale,
         max_num_iterations=o.max_num_iterations, function_tolerance=o.function_tolerance, linear_solver=2,
         **scene_arrays(sc), **{"ref_" + k: v for k, v in r.items()})


def ba_windows(tmp):
    """Local-BA windows of the batched workload (Brown-T2, one intrinsic group,
    cameras 0 and 1 held) at 5, 20 and 40 cameras, solved by ceres
    SPARSE_SCHUR with the call-site options."""
    for cams, pts, seed in ((5, 200, 44), (20, 400, 45), (40, 600, 46)):
        rng = np.random.default_rng(seed)
        sc = scenes.local_problem(rng, cams, pts)
        sc["camera_constant"][1] = 1
        ba_case(tmp, f"window_{cams}", sc, max_num_iterations=100)


def sfm_scans(tmp):
    """The engine-side scans: pair triangulation with the Resection filter
    (residual thresholds 4 px) and the MakeInitialPair3D filter (no residual
    test), the bad-track rejection (precision 4 px) and the residual
    histogram, from the reference's own camera, DLT and histogram code."""
    pr = scenes.engine_pair()
    for name, th in (("resection", 4.0), ("initial", 1e300)):
        r = oracle.ref_run("two-view", {"cameras": pr["cameras"], "x1": pr["x1"], "x2": pr["x2"],
                                        "inlier": pr["inlier"], "max_residual1": th, "max_residual2": th,
                                        "min_angle": 2.0}, tmp)
        save(f"sfm_pair_{name}.npz", max_residual=th, min_angle=2.0, **pr, **{"ref_" + k: v for k, v in r.items()})
    tr = scenes.engine_tracks()
    kv = {k: tr[k] for k in ("cameras", "points", "track_offsets", "camera_index", "xy")}
    r = oracle.ref_run("reject", dict(kv, precision=4.0), tmp)
    h = oracle.ref_run("histogram", kv, tmp)
    save("sfm_tracks.npz", precision=4.0, **tr, **{"ref_" + k: v for k, v in r.items()},
         **{"ref_hist_" + k: v for k, v in h.items()})


def ba_illconditioned(tmp):
    """A scene with ill-conditioned point blocks (twin cameras 0.01 apart,
    40% of the points seen by one twin pair only), solved by ceres to a tight
    tolerance: the minimum the mixed path's precision safeguards must reach."""
    sc = scenes.illconditioned_scene()
    ba_case(tmp, "illconditioned", sc, max_num_iterations=100, function_tolerance=1e-12,
            loss_type=abi.LOSS_HUBER, loss_scale=4.0)


def sfm_pack(tmp):
    """The engine's BA assembly and write-back from its own std::map state,
    with ceres's rotation conversions."""
    st = scenes.engine_state()
    kv = {k: v for k, v in st.items() if k != "intrinsic_group"}
    kv["image_group_key"] = st["group_keys"][st["intrinsic_group"]]
    r = oracle.ref_run("pack", kv, tmp)
    save("sfm_pack.npz", **st, **{"ref_" + k: v for k, v in r.items()})


def sfm_acransac(tmp):
    """robustResection's AC-RANSAC from the reference: the six-point DLT
    kernel (unknown K, 4,096 iterations) and the P3P kernel (known K, 1,024
    iterations), every model drawn recorded with its reference score."""
    sc = scenes.resection_scene()
    base = {"x2d": sc["x2d"], "x3d": sc["x3d"], "width": sc["width"], "height": sc["height"], "seed": 1}
    r = oracle.ref_run("acransac", dict(base, iterations=4096), tmp)
    save("sfm_acransac_6pt.npz", **sc, **{"ref_" + k: v for k, v in r.items()})
    r = oracle.ref_run("acransac", dict(base, iterations=1024, K=sc["K"]), tmp)
    save("sfm_acransac_p3p.npz", **sc, **{"ref_" + k: v for k, v in r.items()})


GENERATORS = {
    "ba_illconditioned": ba_illconditioned,
    "sfm_acransac": sfm_acransac,
    "sfm_pack": sfm_pack,
    "sfm_scans": sfm_scans,
    "tri_ring": lambda tmp: (tri_ring(tmp, 2, 12), tri_ring(tmp, 5, 6)),
    "tri_noisy": tri_noisy,
    "tri_tracks_f32": tri_tracks_f32,
    "tri_long": tri_long,
    "ba_iterative": ba_iterative,
    "ba_windows": ba_windows,
}


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/ref_harness missing: run `make -C oracle ref` first")
    tmp = tempfile.mkdtemp()
    only = sys.argv[1:]
    if only:
        # regenerate the named groups only (python make_golden.py tri_long ba_windows)
        for name in only:
            GENERATORS[name](tmp)
        return
    tri_ring(tmp, 2, 12)
    tri_ring(tmp, 5, 6)
    tri_noisy(tmp)

    # BA problems, each solved by ceres SPARSE_SCHUR/CX_SPARSE with the
    # reference functor of the layout.  With per-camera intrinsics, holding
    # only camera 0 (the incremental engine's gauge) leaves the scale free and
    # the minimum is a flat valley on which two correct LM implementations stop
    # at different points; these scenes also hold camera 1 so that the
    # minimum is isolated and runs to convergence are comparable.
    sc = scenes.ring_scene(num_cameras=16, num_points=300, seed=31)
    ba_case(tmp, "ring_k3_const", sc, max_num_iterations=20)
    sc = scenes.ring_scene(num_cameras=10, num_points=200, seed=32)
    sc["intrinsic_constant"][:] = 0
    sc["intrinsic_fixed_mask"] = 0b111110  # the incremental engine's !refine subset (:1396-1409)
    ba_case(tmp, "ring_k3_focal_huber", sc, max_num_iterations=20, loss_type=abi.LOSS_HUBER, loss_scale=4.0)
    sc = scenes.medium_scene(num_cameras=12, num_points=300, seed=33)
    sc["camera_constant"][1] = 1
    ba_case(tmp, "k3_percam_huber", sc, max_num_iterations=100)
    sc = scenes.medium_scene(num_cameras=8, num_points=200, seed=34, model=abi.BROWN_T2)
    sc["camera_constant"][1] = 1
    ba_case(tmp, "t2_percam_huber", sc, max_num_iterations=100)
    sc = scenes.ring_scene(num_cameras=8, num_points=150, seed=35, model=abi.PINHOLE_F)
    sc["intrinsic_constant"][:] = 0
    ba_case(tmp, "pinhole_f_split", sc, max_num_iterations=20)
    sc = scenes.ring_scene(num_cameras=8, num_points=150, seed=36, model=abi.PINHOLE_F)
    sc["extrinsic_fixed_mask"] = 0b000111  # rotation held: translation-only refinement (:1438)
    ba_case(tmp, "t_only", sc, layout=2, max_num_iterations=20, loss_type=abi.LOSS_HUBER, loss_scale=16.0)
    sc = scenes.ring_scene(num_cameras=8, num_points=150, seed=37, model=abi.PINHOLE_F)
    ba_case(tmp, "rt_only", sc, layout=3, max_num_iterations=20, loss_type=abi.LOSS_HUBER, loss_scale=4.0)
    sc, _ = unit_test_scene(tmp)
    ba_case(tmp, "unit_test_rtf7", sc, layout=1, max_num_iterations=50)

    # Problem::Evaluate at the initial point (Jacobian pins)
    eval_case(tmp, "k3", scenes.medium_scene(num_cameras=4, num_points=15, seed=41), loss=abi.LOSS_HUBER, a=4.0)
    eval_case(tmp, "t2", scenes.medium_scene(num_cameras=4, num_points=15, seed=42, model=abi.BROWN_T2))
    sc = scenes.ring_scene(num_cameras=4, num_points=15, seed=43, model=abi.PINHOLE_F)
    sc["extrinsics"][1, :3] = [1e-9, -2e-9, 5e-10]  # small-angle branch of AngleAxisRotatePoint
    eval_case(tmp, "pinhole_f", sc)
    tri_tracks_f32(tmp)
    tri_long(tmp)
    ba_iterative(tmp)
    ba_windows(tmp)
    sfm_scans(tmp)
    sfm_pack(tmp)
    sfm_acransac(tmp)
    ba_illconditioned(tmp)


if __name__ == "__main__":
    main()
