"""Python access to the CPU oracle (liboracle.so, built from gbba_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline, never by the product package.
"""
import ctypes as C
import importlib
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
