"""Python access to the CPU oracle (liboracle.so, built from gbba_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline, never by the product package.
"""
import ctypes as C
import importlib
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
_lib = None


def reference_dir():
    """Root of the reference's sources, from GBBA_REFERENCE_DIR (the same
    variable the oracle Makefile reads), or None when they are not present."""
    d = os.environ.get("GBBA_REFERENCE_DIR") or _default_reference_dir()
    return d if os.path.isdir(d) else None


def _default_reference_dir():
    # the Makefile's default; the only place besides it that names the path
    out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return out.stdout.strip() if out.returncode == 0 else ""


def _abi():
    return importlib.import_module("3dreconstruction_gb300.abi")


def build():
    subprocess.run(["make", "-C", HERE, "liboracle.so"], check=True, stdout=subprocess.DEVNULL)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        abi = _abi()
        lib = C.CDLL(LIB)
        vp = C.c_void_p
        lib.oracle_ba_solve.argtypes = [C.POINTER(abi.GbbaProblem), C.POINTER(abi.GbbaOptions),
                                        C.POINTER(abi.GbbaSummary), vp, C.c_int, C.c_int]
        lib.oracle_ba_solve.restype = C.c_int
        lib.oracle_ba_evaluate.argtypes = [C.POINTER(abi.GbbaProblem), C.c_int, C.c_double, vp, vp, vp, vp, vp, vp]
        lib.oracle_ba_evaluate.restype = C.c_int
        lib.oracle_tri_dlt2.argtypes = [C.c_int64, vp, vp, C.c_int64, vp, vp, vp, vp]
        lib.oracle_tri_nview.argtypes = [C.c_int, vp, C.c_int64, vp, vp, vp, C.c_int64, vp, vp]
        lib.oracle_tri_linear_gn.argtypes = [vp, vp, vp, vp, C.c_int64, C.c_int, vp, vp, vp]
        lib.oracle_acransac_score.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int64, vp,
                                              vp, C.c_int64, vp, vp, vp, vp, vp, vp]
        lib.oracle_sfm_pack_maps.argtypes = [C.POINTER(abi.GbsfmEngineState), C.c_int64, vp, vp, vp, vp, vp, vp, vp,
                                             vp, C.c_int, vp]
        _lib = lib
    return _lib


def ba_solve(scene, options, num_threads=0, max_costs=1024):
    """Solve a scene with the oracle; returns (summary dict, params dict, iteration costs)."""
    abi = _abi()
    lib = load()
    hp = abi.HostProblem(scene)
    p = hp.struct()
    s = abi.GbbaSummary()
    costs = np.zeros(max_costs)
    st = lib.oracle_ba_solve(C.byref(p), C.byref(options), C.byref(s), costs.ctypes.data, max_costs, num_threads)
    n = s.num_iterations + 1
    return st, s.as_dict(), hp.params(), costs[:min(n, max_costs)]


def ba_evaluate(scene, loss_type=0, loss_scale=1.0):
    abi = _abi()
    lib = load()
    hp = abi.HostProblem(scene)
    p = hp.struct()
    k = abi.MODEL_K[hp.model]
    no, nc, ni, npt = p.num_observations, p.num_cameras, p.num_intrinsics, p.num_points
    cost = np.zeros(1)
    res = np.zeros((no, 2))
    je = np.zeros((no, 2, 6))
    ji = np.zeros((no, 2, k))
    jp = np.zeros((no, 2, 3))
    g = np.zeros(6 * nc + k * ni + 3 * npt)
    lib.oracle_ba_evaluate(C.byref(p), loss_type, loss_scale, cost.ctypes.data, res.ctypes.data,
                           je.ctypes.data, ji.ctypes.data, jp.ctypes.data, g.ctypes.data)
    return {"cost": cost[0], "residuals": res, "jac_extrinsic": je, "jac_intrinsic": ji,
            "jac_point": jp, "gradient": g}


def tri_dlt2(P1, P2, x1, x2, shared=False):
    lib = load()
    n = len(x1)
    P1 = np.ascontiguousarray(P1, np.float64)
    P2 = np.ascontiguousarray(P2, np.float64)
    x1 = np.ascontiguousarray(x1, np.float64)
    x2 = np.ascontiguousarray(x2, np.float64)
    Xh = np.zeros((n, 4))
    Xe = np.zeros((n, 3))
    lib.oracle_tri_dlt2(n, P1.ctypes.data, P2.ctypes.data, 0 if shared else 12, x1.ctypes.data,
                        x2.ctypes.data, Xh.ctypes.data, Xe.ctypes.data)
    return Xh, Xe


def tri_nview(method, P, offsets, cam, xy):
    lib = load()
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 12)
    offsets = np.ascontiguousarray(offsets, np.int64)
    cam = np.ascontiguousarray(cam, np.uint32)
    xy = np.ascontiguousarray(xy, np.float64)
    n = len(offsets) - 1
    X = np.zeros((n, 3 if method == 2 else 4))
    err = np.zeros(n)
    lib.oracle_tri_nview(method, P.ctypes.data, len(P), offsets.ctypes.data, cam.ctypes.data,
                         xy.ctypes.data, n, X.ctypes.data, err.ctypes.data)
    return X, err


def tri_linear_gn(P, offsets, cam, xy, gn_steps=1):
    lib = load()
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 12)
    offsets = np.ascontiguousarray(offsets, np.int64)
    cam = np.ascontiguousarray(cam, np.uint32)
    xy = np.ascontiguousarray(xy, np.float64)
    n = len(offsets) - 1
    X = np.zeros((n, 3))
    st = np.zeros(n, np.uint8)
    md = np.zeros(n)
    lib.oracle_tri_linear_gn(P.ctypes.data, offsets.ctypes.data, cam.ctypes.data, xy.ctypes.data, n,
                             gn_steps, X.ctypes.data, st.ctypes.data, md.ctypes.data)
    return X, st, md


def tri_gn_steps(P, offsets, cam, xy, X0, steps=1, safeguard=False):
    """FP64 Gauss-Newton steps on the reprojection error of each track, from
    the Euclidean points X0 (numpy restatement; the step the triangulation
    paths apply after their linear estimate): H = sum J^T J, g = sum J^T r over
    the track's views, X <- X - H^-1 g.  With safeguard, as the FP32
    production kernel does, a track keeps its X when the step does not lower
    its squared reprojection error."""
    P = np.asarray(P, np.float64).reshape(-1, 3, 4)
    off = np.asarray(offsets, np.int64)
    cam = np.asarray(cam, np.int64)
    xy = np.asarray(xy, np.float64).reshape(-1, 2)
    X = np.array(X0, np.float64, copy=True)
    tr = np.repeat(np.arange(len(off) - 1), np.diff(off))
    for _ in range(steps):
        Pi = P[cam]
        h = np.einsum("nij,nj->ni", Pi[:, :, :3], X[tr]) + Pi[:, :, 3]
        u, v = h[:, 0] / h[:, 2], h[:, 1] / h[:, 2]
        Ju = (Pi[:, 0, :3] - u[:, None] * Pi[:, 2, :3]) / h[:, 2:3]
        Jv = (Pi[:, 1, :3] - v[:, None] * Pi[:, 2, :3]) / h[:, 2:3]
        ru, rv = u - xy[:, 0], v - xy[:, 1]
        H = np.zeros((len(X), 3, 3))
        g = np.zeros((len(X), 3))
        np.add.at(H, tr, Ju[:, :, None] * Ju[:, None, :] + Jv[:, :, None] * Jv[:, None, :])
        np.add.at(g, tr, Ju * ru[:, None] + Jv * rv[:, None])
        Xn = X - np.linalg.solve(H, g[:, :, None])[:, :, 0]
        if safeguard:
            def cost(Y):
                hh = np.einsum("nij,nj->ni", Pi[:, :, :3], Y[tr]) + Pi[:, :, 3]
                e = ((hh[:, :2] / hh[:, 2:3] - xy) ** 2).sum(1)
                out = np.zeros(len(Y))
                np.add.at(out, tr, e)
                return out
            keep = ~(cost(Xn) <= cost(X))
            Xn[keep] = X[keep]
        X = Xn
    return X


# ------------------------------------------------------------ reference harness
def write_kv(path, items):
    with open(path, "w") as f:
        for name, v in items.items():
            a = np.asarray(v, dtype=np.float64).ravel()
            f.write(f"{name} {a.size}\n")
            f.write(" ".join(repr(float(x)) for x in a))
            f.write("\n")


def read_kv(path):
    out = {}
    with open(path) as f:
        toks = f.read().split()
    i = 0
    while i < len(toks):
        name, n = toks[i], int(toks[i + 1])
        out[name] = np.array([float(t) for t in toks[i + 2:i + 2 + n]])
        i += 2 + n
    return out


def ref_available():
    return os.path.exists(REF_HARNESS)


def ref_run(mode, items, tmpdir, extra_args=()):
    """Run the reference harness (compiled from the reference sources)."""
    inp = os.path.join(tmpdir, f"{mode}_in.txt")
    out = os.path.join(tmpdir, f"{mode}_out.txt")
    if items is not None:
        write_kv(inp, items)
        args = [REF_HARNESS, mode, inp, out]
    else:
        args = [REF_HARNESS, mode, *map(str, extra_args), out]
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode not in (0, 1):
        raise RuntimeError(f"ref_harness {mode} failed: {r.stderr[-2000:]}")
    return read_kv(out)


def scene_to_kv(scene, options, layout=0, linear_solver=0, num_threads=1, preconditioner=0):
    """BA problem + options in the harness's input format."""
    model = int(scene["model"])
    d = {
        "model": model, "layout": layout,
        "loss": options.loss_type, "loss_scale": options.loss_scale,
        "extrinsics": scene["extrinsics"], "intrinsics": scene["intrinsics"], "points": scene["points"],
        "observations": scene["observations"], "camera_index": scene["camera_index"],
        "intrinsic_index": scene["intrinsic_index"], "point_index": scene["point_index"],
        "intrinsic_fixed_mask": scene.get("intrinsic_fixed_mask", 0),
        "extrinsic_fixed_mask": scene.get("extrinsic_fixed_mask", 0),
        "linear_solver": linear_solver, "max_num_iterations": options.max_num_iterations,
        "function_tolerance": options.function_tolerance, "gradient_tolerance": options.gradient_tolerance,
        "parameter_tolerance": options.parameter_tolerance, "num_threads": num_threads,
        "preconditioner": preconditioner, "max_linear_solver_iterations": options.max_linear_solver_iterations,
        "eta": options.eta,
    }
    if scene.get("camera_constant") is not None:
        d["camera_constant"] = scene["camera_constant"]
    if scene.get("intrinsic_constant") is not None:
        d["intrinsic_constant"] = scene["intrinsic_constant"]
    return d


# ------------------------------------------------------------ engine-side scans
def _brown(cams, X):
    """BrownPinholeCamera::Project and Depth for rows of cameras (n, 18) and points."""
    R = cams[:, :9].reshape(-1, 3, 3)
    p = np.einsum("nij,nj->ni", R, X) + cams[:, 9:12]
    xe, ye = p[:, 0] / p[:, 2], p[:, 1] / p[:, 2]
    r2 = xe * xe + ye * ye
    rc = 1 + cams[:, 15] * r2 + cams[:, 16] * r2 * r2 + cams[:, 17] * r2 * r2 * r2
    return np.stack([cams[:, 13] + cams[:, 12] * (xe * rc), cams[:, 14] + cams[:, 12] * (ye * rc)], -1), p[:, 2]


def _angle_deg(c):
    return np.degrees(np.arccos(np.clip(c, -1 + 1e-8, 1 - 1e-8)))


def sfm_triangulate_pair(cams, x1, x2, inlier, th1, th2, min_angle):
    """triangulate2View_Vector (sfm_robust.h:152-195) and its callers' keep
    decision (sfm_incremental_engine.cpp:977-1029, 492-533), restated: X by the
    oracle's TriangulateDLT, the mean PinholeCamera residual through P = K[R|t],
    keep = inlier, BrownPinholeCamera residuals below the thresholds, positive
    depths and AngleBetweenRay above min_angle."""
    cams = np.asarray(cams, np.float64).reshape(-1, 18)
    n = len(x1)
    P = []
    for c in cams[:2]:
        K = np.array([[c[12], 0, c[13]], [0, c[12], c[14]], [0, 0, 1.0]])
        P.append(K @ np.concatenate([c[:9].reshape(3, 3), c[9:12, None]], 1))
    _, X = tri_dlt2(P[0].ravel(), P[1].ravel(), x1, x2, shared=True)

    def pin(Pm, x):
        h = X @ Pm[:, :3].T + Pm[:, 3]
        return np.linalg.norm(x - h[:, :2] / h[:, 2:3], axis=1)
    residual = (pin(P[0], x1) + pin(P[1], x2)) / 2.0
    u1, d1 = _brown(np.repeat(cams[:1], n, 0), X)
    u2, d2 = _brown(np.repeat(cams[1:2], n, 0), X)
    r1, r2 = np.linalg.norm(x1 - u1, axis=1), np.linalg.norm(x2 - u2, axis=1)

    def ray(c, x):
        k = np.stack([(x[:, 0] - c[13]) / c[12], (x[:, 1] - c[14]) / c[12], np.ones(len(x))], 1)
        r = k @ c[:9].reshape(3, 3)
        return r / np.linalg.norm(r, axis=1, keepdims=True)
    a, b = ray(cams[0], x1), ray(cams[1], x2)
    mag = np.sqrt((a * a).sum(1) * (b * b).sum(1))
    keep = (np.asarray(inlier) != 0) & (r1 < th1) & (r2 < th2) & (d1 > 0) & (d2 > 0) & \
        (_angle_deg((a * b).sum(1) / mag) > min_angle)
    return X, residual, keep.astype(np.uint8)


def _track_ids(offsets):
    off = np.asarray(offsets, np.int64)
    return np.repeat(np.arange(len(off) - 1), np.diff(off)), off


def sfm_reject_tracks(cams, points, offsets, cam, xy, precision, min_angle=3.0):
    """badTrackRejector (sfm_incremental_engine.cpp:1047-1140), restated."""
    cams = np.asarray(cams, np.float64).reshape(-1, 18)
    tr, off = _track_ids(offsets)
    cam = np.asarray(cam, np.int64)
    X = np.asarray(points, np.float64)[tr]
    u, _ = _brown(cams[cam], X)
    bad = np.linalg.norm(np.asarray(xy) - u, axis=1) > precision
    R = cams[cam, :9].reshape(-1, 3, 3)
    C = -np.einsum("nji,nj->ni", R, cams[cam, 9:12])
    d = X - C
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nt = len(off) - 1
    first = np.full(nt, -1, np.int64)
    order = np.lexsort((cam, tr))  # per track, lowest camera first
    starts = off[:-1][np.diff(off) > 0]
    first[np.diff(off) > 0] = order[starts]
    ang = _angle_deg((d * d[first[tr]]).sum(1))
    ang[np.arange(len(tr)) == first[tr]] = 0.0
    max_angle = np.zeros(nt)
    np.maximum.at(max_angle, tr, ang)
    narrow = max_angle < min_angle
    erase = bad | narrow[tr]
    erased = np.bincount(tr, weights=erase, minlength=nt).astype(np.int64)
    remaining = np.diff(off) - erased
    gone = (erased > 0) & (remaining < 2)
    return (~erase).astype(np.uint8), (~gone).astype(np.uint8), int(erased.sum()), int(gone.sum())


def sfm_residual_histogram(cams, points, offsets, cam, xy):
    """ComputeResidualsHistogram (sfm_incremental_engine.cpp:1550-1616),
    restated: float residuals, MinMaxMeanMedian<float>, Histogram<double>(min, max, 10)."""
    cams = np.asarray(cams, np.float64).reshape(-1, 18)
    tr, off = _track_ids(offsets)
    u, _ = _brown(cams[np.asarray(cam, np.int64)], np.asarray(points, np.float64)[tr])
    res = np.linalg.norm(np.asarray(xy) - u, axis=1).astype(np.float32)
    out = {"count": len(res)}
    if len(res) > 1:
        v = np.sort(res)
        mn, mx = float(v[0]), float(v[-1])
        out.update(min=mn, max=mx, mean=float(np.float32(v.astype(np.float64).sum() / len(v))),
                   median=float(v[len(v) // 2]))
        x = v.astype(np.float64)
        per = 10 / (mx - mn)
        under = x < mn
        b = ((x - mn) * per).astype(np.int64)
        hist = np.bincount(b[(~under) & (b < 10)], minlength=10)[:10]
        out.update(hist=hist, underflow=int(under.sum()), overflow=int(((~under) & (b >= 10)).sum()))
    return out


def rotation_to_angle_axis(R):
    """ceres::RotationMatrixToAngleAxis (include/ceres/rotation.h:357-370):
    RotationMatrixToQuaternion (Shoemake's branches, :312-350) then
    QuaternionToAngleAxis (:266-306), on one row-major 3x3 matrix."""
    R = np.asarray(R, np.float64).reshape(3, 3)
    q = np.zeros(4)
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    if tr >= 0.0:
        s = math.sqrt(tr + 1.0)
        q[0] = 0.5 * s
        s = 0.5 / s
        q[1], q[2], q[3] = (R[2, 1] - R[1, 2]) * s, (R[0, 2] - R[2, 0]) * s, (R[1, 0] - R[0, 1]) * s
    else:
        i = 1 if R[1, 1] > R[0, 0] else 0
        if R[2, 2] > R[i, i]:
            i = 2
        j, k = (i + 1) % 3, (i + 2) % 3
        s = math.sqrt(R[i, i] - R[j, j] - R[k, k] + 1.0)
        q[i + 1] = 0.5 * s
        s = 0.5 / s
        q[0] = (R[k, j] - R[j, k]) * s
        q[j + 1] = (R[j, i] + R[i, j]) * s
        q[k + 1] = (R[k, i] + R[i, k]) * s
    s2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3]
    if s2 > 0.0:
        st, ct = math.sqrt(s2), q[0]
        two_theta = 2.0 * (math.atan2(-st, -ct) if ct < 0.0 else math.atan2(st, ct))
        kk = two_theta / st
    else:
        kk = 2.0
    return q[1:] * kk


def angle_axis_to_rotation(aa):
    """ceres::AngleAxisToRotationMatrix (include/ceres/rotation.h:372-414),
    returned row-major: Rodrigues' formula, first order below theta^2 = eps."""
    w = np.asarray(aa, np.float64)
    th2 = float(w @ w)
    if th2 > np.finfo(np.float64).eps:
        th = math.sqrt(th2)
        wx, wy, wz = w / th
        c, s = math.cos(th), math.sin(th)
        oc = 1.0 - c
        return np.array([[c + wx * wx * oc, wx * wy * oc - wz * s, wy * s + wx * wz * oc],
                         [wz * s + wx * wy * oc, c + wy * wy * oc, -wx * s + wy * wz * oc],
                         [-wy * s + wx * wz * oc, wx * s + wy * wz * oc, c + wz * wz * oc]])
    return np.array([[1.0, -w[2], w[1]], [w[2], 1.0, -w[0]], [-w[1], w[0], 1.0]])


def sfm_pack(st, lock=0):
    """IncrementalReconstructionEngine::BundleAdjustment's assembly
    (sfm_incremental_engine.cpp:1250-1393) over the dense engine state of
    gbsfm_pack_ba: cameras in ascending image id, observations of the
    reconstructed images in track-major order, and the locked block
    (:1437-1443: camera_index_extrinsic[ordinal of the first-added image])."""
    rec = np.asarray(st["reconstructed"]) != 0
    ordinal = np.cumsum(rec) - 1
    cams = np.asarray(st["cameras"], np.float64).reshape(-1, 18)
    ext = np.array([np.concatenate([rotation_to_angle_axis(cams[i, :9]), cams[i, 9:12]])
                    for i in np.flatnonzero(rec)]).reshape(-1, 6)
    off = np.asarray(st["track_offsets"], np.int64)
    tr = np.repeat(np.arange(len(off) - 1), np.diff(off))
    img = np.asarray(st["track_image"], np.int64)
    keep = rec[img]
    fidx = np.asarray(st["feature_offsets"], np.int64)[img] + np.asarray(st["track_feature"], np.int64)
    obs = np.asarray(st["features"], np.float32)[fidx].astype(np.float64)[keep]
    out = {"extrinsics": ext, "observations": obs, "camera_index": ordinal[img][keep].astype(np.uint32),
           "intrinsic_index": np.asarray(st["intrinsic_group"], np.uint32)[img][keep],
           "point_index": tr[keep].astype(np.uint32), "camera_image": np.flatnonzero(rec).astype(np.uint32),
           "num_cameras": int(rec.sum()), "measurements": len(img)}
    fa = int(st["first_added"])
    locked = -1
    if fa >= 0 and rec.any() and lock != 2:
        k = int(ordinal[fa]) if rec[fa] else (0 if lock == 0 else -1)
        if lock == 1:
            locked = k
        elif k < len(out["camera_index"]):
            locked = int(out["camera_index"][k])
    out["locked_camera"] = locked
    return out


def sfm_unpack(extrinsics, camera_image, intrinsics, intrinsic_group, cameras):
    """The write-back of BundleAdjustment (sfm_incremental_engine.cpp:
    1491-1516): each camera rebuilt from its refined angle-axis, translation
    and its group's intrinsics; rows of the engine camera layout."""
    out = np.array(cameras, np.float64).reshape(-1, 18)
    ext = np.asarray(extrinsics, np.float64).reshape(-1, 6)
    intr = np.asarray(intrinsics, np.float64).reshape(-1, 6)
    for c, i in enumerate(np.asarray(camera_image, np.int64)):
        out[i, :9] = angle_axis_to_rotation(ext[c, :3]).ravel()
        out[i, 9:12] = ext[c, 3:]
        out[i, 12:18] = intr[int(intrinsic_group[i])]
    return out


def sfm_pack_maps(st, repeats=1):
    """The same assembly run by C++ over std::map containers built from the
    state, as the engine runs it (liboracle.so); returns (result dict, mean
    seconds of the assembly loop)."""
    abi = _abi()
    lib = load()
    ep = abi.EnginePack(st)
    s = ep.state_struct()
    ni, ne = ep.ni, ep.ne
    ext = np.zeros((max(ni, 1), 6))
    intr = np.zeros((max(ep.ng, 1), 6))
    pts = np.zeros((max(ep.nt, 1), 3))
    obs = np.zeros((max(ne, 1), 2))
    idx = [np.zeros(max(ne, 1), np.uint32) for _ in range(3)]
    counts = np.zeros(3, np.int64)
    sec = np.zeros(1)
    lib.oracle_sfm_pack_maps(C.byref(s), int(st["first_added"]), ext.ctypes.data, intr.ctypes.data, pts.ctypes.data,
                             obs.ctypes.data, idx[0].ctypes.data, idx[1].ctypes.data, idx[2].ctypes.data,
                             counts.ctypes.data, int(repeats), sec.ctypes.data)
    nc, no = int(counts[0]), int(counts[1])
    return ({"extrinsics": ext[:nc], "intrinsics": intr[:ep.ng], "points": pts[:ep.nt], "observations": obs[:no],
             "camera_index": idx[0][:no], "intrinsic_index": idx[1][:no], "point_index": idx[2][:no],
             "num_cameras": nc, "locked_camera": int(counts[2])}, float(sec[0]))


def _logcombi(k, n):
    """logcombi (estimator_acransac.h:40-49)."""
    if k >= n or k <= 0:
        return 0.0
    if n - k < k:
        k = n - k
    r = 0.0
    for i in range(1, k + 1):
        r += math.log10(n - i + 1) - math.log10(i)
    return r


def acransac_tables(n, sample_size):
    """makelogcombi_n / makelogcombi_k (estimator_acransac.h:52-65), float32."""
    return (np.array([_logcombi(k, n) for k in range(n + 1)], np.float32),
            np.array([_logcombi(sample_size, m) for m in range(n + 1)], np.float32))


def acransac_score(x2d, x3d, models, sample_size, max_models, logalpha0, mult_error=1.0,
                   max_threshold=math.inf, tables=None):
    """The per-model scoring of ACRANSAC's main loop (estimator_acransac.h:
    170-200) on normalised points: ResectionSquaredResidualError
    (sfm_robust.h:197-204), std::sort of (error, index), bestNFA (:75-97).
    Returns nfa, k, e[k-1] per model and the sorted index order."""
    x2d = np.asarray(x2d, np.float64).reshape(-1, 2)
    X = np.asarray(x3d, np.float64).reshape(-1, 3)
    n = len(x2d)
    logc_n, logc_k = tables if tables is not None else acransac_tables(n, sample_size)
    loge0 = math.log10(max_models * (n - sample_size))
    M = np.asarray(models, np.float64).reshape(-1, 3, 4)
    nfa, kk, emax, order = [], [], [], []
    fmin = float(np.finfo(np.float32).tiny)
    for P in M:
        h = X @ P[:, :3].T + P[:, 3]
        d = h[:, :2] / h[:, 2:] - x2d
        e = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]
        o = np.lexsort((np.arange(n), e))
        es = e[o]
        ks = np.arange(sample_size + 1, n + 1)
        ok = np.cumprod(es[ks - 1] <= max_threshold).astype(bool)
        ks = ks[ok]
        v = loge0 + (logalpha0 + mult_error * np.log10(es[ks - 1] + fmin)) * (ks - sample_size) \
            + logc_n[ks].astype(np.float64) + logc_k[ks].astype(np.float64)
        if len(v) and np.min(v) < math.inf:
            j = int(np.argmin(v))
            nfa.append(float(v[j]))
            kk.append(int(ks[j]))
            emax.append(float(es[ks[j] - 1]))
        else:
            nfa.append(math.inf)
            kk.append(sample_size)
            emax.append(math.inf)
        order.append(o)
    return np.array(nfa), np.array(kk), np.array(emax), np.array(order)


def acransac_replay(nfa, k, emax, order, models_per_fit, normalizer):
    """ACRANSAC's model selection (estimator_acransac.h:172-244) over scored
    models in the order they were drawn: a model strictly below the running
    minimum NFA becomes the result; no result unless the minimum is below 0.
    Returns (error_max unnormalised, min_nfa, inliers, model index)."""
    min_nfa, best = math.inf, -1
    m = 0
    for cnt in np.asarray(models_per_fit, np.int64):
        for _ in range(int(cnt)):
            if nfa[m] < min_nfa:
                min_nfa, best = nfa[m], m
            m += 1
    if best < 0:
        return math.inf, min_nfa, np.zeros(0, np.int64), -1
    inliers = np.asarray(order[best][:int(k[best])], np.int64)
    if min_nfa >= 0:
        inliers = inliers[:0]
    err = math.sqrt(emax[best]) / normalizer if len(inliers) else emax[best]
    return err, min_nfa, inliers, best


def acransac_score_cpp(x2d, x3d, models, sample_size, max_models, logalpha0, mult_error=1.0,
                       max_threshold=math.inf, with_order=True):
    """The same scoring in C++ (liboracle), model after model with std::sort;
    returns (nfa, k, e[k-1], order or None, mean seconds per model)."""
    lib = load()
    x2d = np.ascontiguousarray(x2d, np.float64)
    x3d = np.ascontiguousarray(x3d, np.float64)
    models = np.ascontiguousarray(models, np.float64)
    n, h = len(x2d.reshape(-1, 2)), len(models.reshape(-1, 12))
    nfa, emax = np.zeros(h), np.zeros(h)
    k = np.zeros(h, np.int32)
    order = np.zeros((h, n), np.uint32) if with_order else None
    sec = np.zeros(1)
    lib.oracle_acransac_score(sample_size, max_models, logalpha0, mult_error, max_threshold, n, x2d.ctypes.data,
                              x3d.ctypes.data, h, models.ctypes.data, nfa.ctypes.data, k.ctypes.data,
                              emax.ctypes.data, order.ctypes.data if with_order else None, sec.ctypes.data)
    return nfa, k, emax, order, float(sec[0])
