"""Seeded synthetic scenes for the bundle-adjustment and triangulation path.

The reference publishes no dataset for this path; its tests use synthetic
ring scenes (libs/multiview/src/nview_data_sets.cpp:23-66).  These generators
produce the five workloads the engine is measured on, with numpy's PCG64
generator seeded per scene (seed = workload number unless given):

  ring16      16 cameras on a ring of radius 10 (XZ plane, Y up) looking at
              the origin through the reference's LookAt (libs/base/src/math/
              numeric.cpp:44), f=1000, pp=(960,540), 2,000 points in
              [-2,2]^3, pixel noise 0.5, poses perturbed 0.01 rad / 0.05,
              points by N(0,0.05^2); camera 0 and the shared intrinsics held.
  tracks1m    200 cameras on a sphere of radius 15, f~U[800,1200], 1,000,000
              points in [-3,3]^3, track length U{2..30}, noise 1 px.
  medium      500 cameras with per-camera radial-K3 intrinsics, 200,000
              points, views Poisson(8)+2, noise 0.7 px + 5% outliers, Huber 4.
  local4096   4,096 independent local problems, 5-40 cameras and 200-5,000
              points each, Brown-T2 intrinsics shared inside a problem.
  large       5,000 cameras K3, 2,000,000 points, views Geometric(mean 10,
              min 2), noise 0.5 px + 2% outliers, Huber.
"""
import math

import numpy as np

from . import abi

IMAGE_W, IMAGE_H = 1920.0, 1080.0
PP = (960.0, 540.0)


# ----------------------------------------------------------------- geometry
def look_at(direction, up=(0.0, 1.0, 0.0)):
    """Rows x_c, y_c, z_c with z_c along `direction` (numeric.cpp:44-52)."""
    zc = np.asarray(direction, dtype=np.float64)
    zc = zc / np.linalg.norm(zc, axis=-1, keepdims=True)
    up = np.broadcast_to(np.asarray(up, dtype=np.float64), zc.shape)
    xc = np.cross(up, zc)
    xc = xc / np.linalg.norm(xc, axis=-1, keepdims=True)
    yc = np.cross(zc, xc)
    return np.stack([xc, yc, zc], axis=-2)


def rotation_to_angle_axis(R):
    """Angle-axis of rotation matrices (batched); the scenes keep angles < pi."""
    R = np.asarray(R, dtype=np.float64)
    tr = np.clip((np.trace(R, axis1=-2, axis2=-1) - 1.0) / 2.0, -1.0, 1.0)
    theta = np.arccos(tr)
    w = np.stack([R[..., 2, 1] - R[..., 1, 2], R[..., 0, 2] - R[..., 2, 0], R[..., 1, 0] - R[..., 0, 1]], -1)
    s = np.sin(theta)
    small = s < 1e-12
    factor = np.where(small, 0.5, theta / (2.0 * np.where(small, 1.0, s)))
    return w * factor[..., None]


def angle_axis_to_rotation(w):
    w = np.asarray(w, dtype=np.float64)
    theta = np.linalg.norm(w, axis=-1)
    safe = np.where(theta > 1e-15, theta, 1.0)
    k = w / safe[..., None]
    K = np.zeros(w.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2] = -k[..., 2], k[..., 1]
    K[..., 1, 0], K[..., 1, 2] = k[..., 2], -k[..., 0]
    K[..., 2, 0], K[..., 2, 1] = -k[..., 1], k[..., 0]
    s, c = np.sin(theta)[..., None, None], np.cos(theta)[..., None, None]
    I = np.broadcast_to(np.eye(3), K.shape)
    return I + s * K + (1 - c) * (K @ K)


def project(model, intr, ext, X):
    """Predicted pixels for rows of (intrinsics, extrinsics, points)."""
    R = angle_axis_to_rotation(ext[:, :3])
    p = np.einsum("nij,nj->ni", R, X) + ext[:, 3:6]
    x, y = p[:, 0] / p[:, 2], p[:, 1] / p[:, 2]
    if model == abi.PINHOLE_F:
        return np.stack([intr[:, 0] * x, intr[:, 0] * y], -1), p[:, 2]
    r2 = x * x + y * y
    rc = 1 + intr[:, 3] * r2 + intr[:, 4] * r2 * r2 + intr[:, 5] * r2 * r2 * r2
    xd, yd = x * rc, y * rc
    if model == abi.BROWN_T2:
        xd = xd + 2 * intr[:, 6] * x * y + intr[:, 7] * (r2 + 2 * x * x)
        yd = yd + 2 * intr[:, 7] * x * y + intr[:, 6] * (r2 + 2 * y * y)
    return np.stack([intr[:, 1] + intr[:, 0] * xd, intr[:, 2] + intr[:, 0] * yd], -1), p[:, 2]


def sphere_directions(n, rng, max_elevation_deg=60.0):
    """Roughly uniform directions, elevation limited so LookAt's up stays valid."""
    i = np.arange(n) + 0.5
    ymax = math.sin(math.radians(max_elevation_deg))
    y = ymax * (1 - 2 * i / n)
    phi = i * math.pi * (3.0 - math.sqrt(5.0)) + rng.uniform(0, 2 * math.pi)
    r = np.sqrt(1 - y * y)
    return np.stack([r * np.cos(phi), y, r * np.sin(phi)], -1)


def _cameras_facing_origin(centers):
    R = look_at(-centers)
    t = -np.einsum("nij,nj->ni", R, centers)
    return R, t


def _perturb(rng, ext, points, rot_sigma, t_sigma, x_sigma, fixed_cams=()):
    ext0 = ext.copy()
    axis = rng.normal(size=(ext.shape[0], 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    ext[:, :3] += rot_sigma * axis
    d = rng.normal(size=(ext.shape[0], 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ext[:, 3:] += t_sigma * d
    for c in fixed_cams:
        ext[c] = ext0[c]
    points = points + rng.normal(scale=x_sigma, size=points.shape)
    return ext, points


def _scene_dict(model, ext, intr, pts, obs, cam, intr_idx, pt_idx, **extra):
    d = {
        "model": model,
        "extrinsics": np.ascontiguousarray(ext, dtype=np.float64),
        "intrinsics": np.ascontiguousarray(intr, dtype=np.float64),
        "points": np.ascontiguousarray(pts, dtype=np.float64),
        "observations": np.ascontiguousarray(obs, dtype=np.float64),
        "camera_index": np.ascontiguousarray(cam, dtype=np.uint32),
        "intrinsic_index": np.ascontiguousarray(intr_idx, dtype=np.uint32),
        "point_index": np.ascontiguousarray(pt_idx, dtype=np.uint32),
    }
    d.update(extra)
    return d


def _observe(rng, model, ext_true, intr_true, X_true, cam, intr_idx, pt, sigma, outlier_frac=0.0):
    pred, depth = project(model, intr_true[intr_idx], ext_true[cam], X_true[pt])
    obs = pred + rng.normal(scale=sigma, size=pred.shape)
    if outlier_frac > 0:
        m = rng.random(len(obs)) < outlier_frac
        obs[m, 0] = rng.uniform(0, IMAGE_W, m.sum())
        obs[m, 1] = rng.uniform(0, IMAGE_H, m.sum())
    return obs, pred, depth


# ----------------------------------------------------------------- workloads
def ring_scene(num_cameras=16, num_points=2000, seed=1, radius=10.0, extent=2.0, sigma=0.5,
               rot_sigma=0.01, t_sigma=0.05, x_sigma=0.05, model=abi.RADIAL_K3):
    """The small plain-FP64 scene (ring of cameras, shared constant intrinsics)."""
    rng = np.random.default_rng(seed)
    theta = np.arange(num_cameras) * 2 * math.pi / num_cameras
    centers = radius * np.stack([np.sin(theta), np.zeros_like(theta), np.cos(theta)], -1)
    R, t = _cameras_facing_origin(centers)
    ext_true = np.concatenate([rotation_to_angle_axis(R), t], 1)
    if model == abi.PINHOLE_F:
        intr = np.array([[1000.0]])
    else:
        intr = np.zeros((1, abi.MODEL_K[model]))
        intr[0, :3] = (1000.0, PP[0], PP[1])
    X_true = rng.uniform(-extent, extent, size=(num_points, 3))
    pt = np.repeat(np.arange(num_points), num_cameras)
    cam = np.tile(np.arange(num_cameras), num_points)
    intr_idx = np.zeros_like(cam)
    pred, depth = project(model, intr[intr_idx], ext_true[cam], X_true[pt])
    inside = (depth > 0) & (pred[:, 0] >= 0) & (pred[:, 0] < IMAGE_W) & (pred[:, 1] >= 0) & (pred[:, 1] < IMAGE_H)
    if model == abi.PINHOLE_F:
        inside = depth > 0
    pt, cam, intr_idx = pt[inside], cam[inside], intr_idx[inside]
    obs, _, _ = _observe(rng, model, ext_true, intr, X_true, cam, intr_idx, pt, sigma)
    ext, pts = _perturb(rng, ext_true.copy(), X_true, rot_sigma, t_sigma, x_sigma, fixed_cams=(0,))
    cam_const = np.zeros(num_cameras, np.uint8)
    cam_const[0] = 1
    return _scene_dict(model, ext, intr, pts, obs, cam, intr_idx, pt,
                       camera_constant=cam_const, intrinsic_constant=np.ones(1, np.uint8),
                       truth={"extrinsics": ext_true, "points": X_true, "intrinsics": intr.copy()},
                       name="ring16", seed=seed)


def medium_scene(num_cameras=500, num_points=200_000, seed=3, mean_views=8, sigma=0.7,
                 outlier_frac=0.05, huber=4.0, rot_sigma=0.01, t_sigma=0.05, x_sigma=0.05,
                 k_sigma=(0.05, 0.01, 0.01), radius=15.0, extent=3.0, model=abi.RADIAL_K3,
                 geometric_views=False, hold=(0,)):
    """Per-camera radial-K3 (or Brown-T2) scene with outliers under a Huber loss.

    `hold` lists the cameras whose extrinsics are held constant: camera 0 is
    the reference's gauge; holding a second camera also fixes the scale, so
    that the minimum is isolated instead of a flat valley."""
    rng = np.random.default_rng(seed)
    centers = radius * sphere_directions(num_cameras, rng)
    R, t = _cameras_facing_origin(centers)
    ext_true = np.concatenate([rotation_to_angle_axis(R), t], 1)
    k = abi.MODEL_K[model]
    intr_true = np.zeros((num_cameras, k))
    intr_true[:, 0] = rng.uniform(900, 1100, num_cameras)
    intr_true[:, 1], intr_true[:, 2] = PP
    if k >= 6:
        intr_true[:, 3] = rng.normal(0, k_sigma[0], num_cameras)
        intr_true[:, 4] = rng.normal(0, k_sigma[1], num_cameras)
        intr_true[:, 5] = rng.normal(0, k_sigma[2], num_cameras)
    if k == 8:
        intr_true[:, 6:8] = rng.normal(0, 0.002, (num_cameras, 2))
    X_true = rng.uniform(-extent, extent, size=(num_points, 3))
    if geometric_views:
        views = 2 + rng.geometric(1.0 / (mean_views - 1), num_points) - 1
    else:
        views = rng.poisson(mean_views, num_points) + 2
    views = np.minimum(views, num_cameras)
    pt = np.repeat(np.arange(num_points), views)
    # distinct cameras per point: start + j*step (mod C) with step coprime to C
    start = rng.integers(0, num_cameras, num_points)
    steps = np.array([s for s in range(1, num_cameras) if math.gcd(s, num_cameras) == 1])
    step = steps[rng.integers(0, len(steps), num_points)]
    j = np.arange(len(pt)) - np.repeat(np.cumsum(views) - views, views)
    cam = (np.repeat(start, views) + j * np.repeat(step, views)) % num_cameras
    order = np.lexsort((cam, pt))
    pt, cam = pt[order], cam[order]
    intr_idx = cam.copy()
    obs, pred, depth = _observe(rng, model, ext_true, intr_true, X_true, cam, intr_idx, pt, sigma, outlier_frac)
    ext, pts = _perturb(rng, ext_true.copy(), X_true, rot_sigma, t_sigma, x_sigma, fixed_cams=tuple(hold))
    intr = intr_true.copy()
    intr[:, 0] *= 1 + rng.normal(0, 0.002, num_cameras)
    cam_const = np.zeros(num_cameras, np.uint8)
    cam_const[list(hold)] = 1
    return _scene_dict(model, ext, intr, pts, obs, cam, intr_idx, pt,
                       camera_constant=cam_const, loss=abi.LOSS_HUBER, loss_scale=huber,
                       truth={"extrinsics": ext_true, "points": X_true, "intrinsics": intr_true},
                       name="medium", seed=seed)


def large_scene(seed=5, **kw):
    args = dict(num_cameras=5000, num_points=2_000_000, mean_views=10, sigma=0.5,
                outlier_frac=0.02, geometric_views=True)
    args.update(kw)
    s = medium_scene(seed=seed, **args)
    s["name"] = "large"
    return s


def local_problem(rng, num_cameras, num_points, model=abi.BROWN_T2, sigma=0.5, rot_sigma=0.02,
                  t_sigma=0.05, x_sigma=0.05, radius=8.0, extent=2.0, num_groups=1):
    """One local-BA window: cameras on an arc sharing one intrinsic group, or
    `num_groups` groups assigned to the cameras round robin (camera c uses
    group c % num_groups)."""
    ang = np.linspace(-0.6, 0.6, num_cameras) + rng.uniform(-0.05, 0.05, num_cameras)
    centers = radius * np.stack([np.sin(ang), rng.uniform(-0.1, 0.1, num_cameras), np.cos(ang)], -1)
    R, t = _cameras_facing_origin(centers)
    ext_true = np.concatenate([rotation_to_angle_axis(R), t], 1)
    k = abi.MODEL_K[model]
    intr_true = np.zeros((num_groups, k))
    for g in range(num_groups):
        intr_true[g, :3] = (rng.uniform(900, 1100), PP[0], PP[1])
        if k >= 6:
            intr_true[g, 3:6] = rng.normal(0, (0.05, 0.01, 0.01))
        if k == 8:
            intr_true[g, 6:8] = rng.normal(0, 0.002, 2)
    X_true = rng.uniform(-extent, extent, size=(num_points, 3))
    views = rng.integers(2, num_cameras + 1, num_points)
    pt = np.repeat(np.arange(num_points), views)
    start = rng.integers(0, num_cameras, num_points)
    steps = np.array([s for s in range(1, num_cameras) if math.gcd(s, num_cameras) == 1])
    step = steps[rng.integers(0, len(steps), num_points)]
    j = np.arange(len(pt)) - np.repeat(np.cumsum(views) - views, views)
    cam = (np.repeat(start, views) + j * np.repeat(step, views)) % num_cameras
    order = np.lexsort((cam, pt))
    pt, cam = pt[order], cam[order]
    intr_idx = cam % num_groups
    obs, _, _ = _observe(rng, model, ext_true, intr_true, X_true, cam, intr_idx, pt, sigma)
    ext, pts = _perturb(rng, ext_true.copy(), X_true, rot_sigma, t_sigma, x_sigma, fixed_cams=(0,))
    intr = intr_true.copy()
    if num_groups == 1:
        intr[0, 0] *= 1 + rng.normal(0, 0.002)
    else:
        intr[:, 0] *= 1 + rng.normal(0, 0.002, num_groups)
    cam_const = np.zeros(num_cameras, np.uint8)
    cam_const[0] = 1
    return _scene_dict(model, ext, intr, pts, obs, cam, intr_idx, pt, camera_constant=cam_const)


def local_batch(num_problems=4096, seed=4, cams=(5, 40), points=(200, 5000), model=abi.BROWN_T2):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(num_problems):
        c = int(rng.integers(cams[0], cams[1] + 1))
        p = int(rng.integers(points[0], points[1] + 1))
        out.append(local_problem(rng, c, p, model=model))
    return out


def local_window(seed, index, cams=(5, 40), points=(200, 5000), model=abi.BROWN_T2, hold_second=True):
    """Window `index` of the batched local-BA workload, from its own seeded
    generator (so that windows can be generated in parallel): cameras uniform
    in `cams`, points uniform in `points`, one Brown-T2 intrinsic group.  With
    hold_second, camera 1 is held besides the gauge camera 0, which fixes the
    scale so that each window's minimum is isolated."""
    rng = np.random.default_rng([seed, index])
    c = int(rng.integers(cams[0], cams[1] + 1))
    p = int(rng.integers(points[0], points[1] + 1))
    prob = local_problem(rng, c, p, model=model)
    if hold_second:
        prob["camera_constant"][1] = 1
    return prob


def track_scene(num_cameras=200, num_tracks=1_000_000, seed=2, radius=15.0, extent=3.0, sigma=1.0,
                min_len=2, max_len=30, f_range=(800.0, 1200.0)):
    """Batched-triangulation workload: tracks as CSR over a camera table."""
    rng = np.random.default_rng(seed)
    centers = radius * sphere_directions(num_cameras, rng)
    R, t = _cameras_facing_origin(centers)
    f = rng.uniform(f_range[0], f_range[1], num_cameras)
    K = np.zeros((num_cameras, 3, 3))
    K[:, 0, 0] = f
    K[:, 1, 1] = f
    K[:, 0, 2], K[:, 1, 2] = PP
    K[:, 2, 2] = 1
    P = np.einsum("nij,njk->nik", K, np.concatenate([R, t[:, :, None]], 2))
    X = rng.uniform(-extent, extent, size=(num_tracks, 3))
    L = rng.integers(min_len, max_len + 1, num_tracks)
    L = np.minimum(L, num_cameras)
    tr = np.repeat(np.arange(num_tracks), L)
    start = rng.integers(0, num_cameras, num_tracks)
    steps = np.array([s for s in range(1, num_cameras) if math.gcd(s, num_cameras) == 1])
    step = steps[rng.integers(0, len(steps), num_tracks)]
    j = np.arange(len(tr)) - np.repeat(np.cumsum(L) - L, L)
    cam = (np.repeat(start, L) + j * np.repeat(step, L)) % num_cameras
    Xh = np.concatenate([X[tr], np.ones((len(tr), 1))], 1)
    h = np.einsum("nij,nj->ni", P[cam], Xh)
    xy = h[:, :2] / h[:, 2:3] + rng.normal(scale=sigma, size=(len(tr), 2))
    offsets = np.zeros(num_tracks + 1, np.int64)
    offsets[1:] = np.cumsum(L)
    return {"P": np.ascontiguousarray(P.reshape(num_cameras, 12)), "track_offsets": offsets,
            "camera_index": cam.astype(np.uint32), "xy": np.ascontiguousarray(xy), "X_true": X,
            "name": "tracks1m", "seed": seed}


def ba_options_for(scene, **kw):
    """Solver options of the reference call sites for a scene (loss from the scene)."""
    o = abi.default_options()
    o.loss_type = int(scene.get("loss", abi.LOSS_SQUARED))
    o.loss_scale = float(scene.get("loss_scale", 1.0))
    for key, v in kw.items():
        setattr(o, key, v)
    return o


# ----------------------------------------------------------------- engine-side scans
def brown_cameras(centers, rng, k_sigma=(0.05, 0.01, 0.01), f_range=(900.0, 1100.0)):
    """Cameras in the layout of the engine's BrownPinholeCamera: rows of
    [R (row-major 9), t (3), f, ppx, ppy, k1, k2, k3], facing the origin."""
    R, t = _cameras_facing_origin(centers)
    n = len(centers)
    cams = np.zeros((n, 18))
    cams[:, :9] = R.reshape(n, 9)
    cams[:, 9:12] = t
    cams[:, 12] = rng.uniform(f_range[0], f_range[1], n)
    cams[:, 13], cams[:, 14] = PP
    cams[:, 15:18] = rng.normal(0, k_sigma, (n, 3))
    return cams


def brown_project(cams, X):
    """Pixels of X through the cameras (rows paired): R X + t, x/z, the radial
    K3 factor, f and the principal point; and the depth."""
    R = cams[:, :9].reshape(-1, 3, 3)
    p = np.einsum("nij,nj->ni", R, X) + cams[:, 9:12]
    x, y = p[:, 0] / p[:, 2], p[:, 1] / p[:, 2]
    r2 = x * x + y * y
    rc = 1 + cams[:, 15] * r2 + cams[:, 16] * r2 * r2 + cams[:, 17] * r2 * r2 * r2
    return np.stack([cams[:, 13] + cams[:, 12] * x * rc, cams[:, 14] + cams[:, 12] * y * rc], -1), p[:, 2]


def engine_pair(n=2000, seed=7, baseline=1.5, sigma=0.5, outlier_frac=0.05, far_frac=0.1, behind_frac=0.05):
    """Matches between two cameras for the engine's pair triangulation: points
    in front of both, a share far away (small ray angles), a share behind, and
    outliers; an inlier mask of the caller's robust estimation (90%)."""
    rng = np.random.default_rng(seed)
    centers = np.array([[-baseline / 2, 0.0, -10.0], [baseline / 2, 0.0, -10.0]])
    cams = brown_cameras(centers, rng)
    X = rng.uniform(-2, 2, (n, 3))
    far = rng.random(n) < far_frac
    X[far, 2] += rng.uniform(60, 200, far.sum())
    behind = rng.random(n) < behind_frac
    X[behind, 2] = -25.0 + rng.uniform(-2, 2, behind.sum())
    x1, _ = brown_project(np.repeat(cams[:1], n, 0), X)
    x2, _ = brown_project(np.repeat(cams[1:], n, 0), X)
    x1 += rng.normal(scale=sigma, size=x1.shape)
    x2 += rng.normal(scale=sigma, size=x2.shape)
    out = rng.random(n) < outlier_frac
    x2[out] += rng.normal(scale=25.0, size=(out.sum(), 2))
    inlier = (rng.random(n) < 0.9).astype(np.uint8)
    return {"cameras": cams, "x1": x1, "x2": x2, "inlier": inlier}


def engine_tracks(num_cameras=30, num_tracks=3000, seed=8, sigma=0.5, outlier_frac=0.03, narrow_frac=0.05,
                  max_len=10, twins=6):
    """Reconstructed tracks for the engine's bad-track rejection and residual
    statistics: CSR over cameras (observations of a track in increasing camera
    order), one 3D point per track, lengths 1..max_len, pixel noise and
    outliers.  The last `twins` cameras sit 0.3 units from the first ones, and
    a share of the tracks is seen only by such a pair, so that their rays meet
    at small angles."""
    rng = np.random.default_rng(seed)
    centers = 12.0 * sphere_directions(num_cameras, rng)
    tang = np.cross(centers[:twins], np.array([0.0, 1.0, 0.0]))
    tang /= np.linalg.norm(tang, axis=1, keepdims=True)
    centers = np.concatenate([centers, centers[:twins] + 0.3 * tang])
    cams = brown_cameras(centers, rng)
    X = rng.uniform(-2, 2, (num_tracks, 3))
    narrow = rng.random(num_tracks) < narrow_frac
    L = rng.integers(1, max_len + 1, num_tracks)
    L[narrow] = 2
    groups = []
    for t in range(num_tracks):
        if narrow[t]:
            k = int(rng.integers(0, twins))
            groups.append(np.array([k, num_cameras + k]))
        else:
            groups.append(np.sort(rng.choice(num_cameras, L[t], replace=False)))
    cam = np.concatenate(groups).astype(np.uint32)
    tr = np.repeat(np.arange(num_tracks), L)
    xy, _ = brown_project(cams[cam], X[tr])
    xy += rng.normal(scale=sigma, size=xy.shape)
    out = rng.random(len(tr)) < outlier_frac
    xy[out] += rng.normal(scale=20.0, size=(out.sum(), 2))
    off = np.zeros(num_tracks + 1, np.int64)
    off[1:] = np.cumsum(L)
    return {"cameras": cams, "points": X, "track_offsets": off, "camera_index": cam, "xy": xy}


def _axis_rotation(axis, angle):
    """Rotation matrix of `angle` about the unit `axis` (Rodrigues)."""
    k = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * (K @ K)


def engine_state(num_images=40, num_points=2000, seed=9, reconstructed_frac=0.8, num_groups=3, max_len=8):
    """The incremental engine's state before a bundle adjustment, as dense
    arrays in the key order of its maps: cameras per image (some images not
    reconstructed), intrinsic groups with non-dense keys, features per image
    (float pixels), 3D points with non-dense track ids, and tracks whose
    entries (image, feature) ascend by image and may name images without a
    camera.  A few rotations take the special branches of the matrix to
    angle-axis conversion: the identity, half turns about each axis, a turn
    just short of half, and a small angle.  Also a refined parameter set for
    the write-back: angle-axis vectors of zero, sub-epsilon, near-pi and
    generic length."""
    rng = np.random.default_rng(seed)
    centers = 12.0 * sphere_directions(num_images, rng)
    cams = brown_cameras(centers, rng)
    special = [np.eye(3), _axis_rotation([1, 0, 0], math.pi), _axis_rotation([0, 1, 0], math.pi),
               _axis_rotation([0, 0, 1], math.pi), _axis_rotation([1, 2, -1], math.pi - 1e-3),
               _axis_rotation([0.3, -1, 0.2], 1e-6), _axis_rotation([-2, 1, 3], 2.5)]
    slots = [3 + 2 * i for i in range(len(special)) if 3 + 2 * i < num_images]
    for i, R in zip(slots, special):
        cams[i, :9] = R.ravel()
    rec = (rng.random(num_images) < reconstructed_frac).astype(np.uint8)
    rec[slots] = 1
    group_keys = np.sort(rng.choice(np.arange(2, 40), num_groups, replace=False))
    image_group = rng.integers(0, num_groups, num_images).astype(np.uint32)
    group_intr = np.column_stack([rng.uniform(900, 1100, num_groups), np.full(num_groups, PP[0]),
                                  np.full(num_groups, PP[1]), rng.normal(0, 0.05, num_groups),
                                  rng.normal(0, 0.01, num_groups), rng.normal(0, 0.01, num_groups)])
    nfeat = rng.integers(20, 400, num_images)
    nfeat[0] = 0  # an image without features, named by no track
    feature_offsets = np.zeros(num_images + 1, np.int64)
    feature_offsets[1:] = np.cumsum(nfeat)
    features = rng.uniform(0, 2000, (int(feature_offsets[-1]), 2)).astype(np.float32)
    track_keys = np.sort(rng.choice(np.arange(10 * num_points), num_points, replace=False)).astype(np.int64)
    X = rng.uniform(-2, 2, (num_points, 3))
    L = rng.integers(2, max_len + 1, num_points)
    L[5] = 1
    imgs, fts = [], []
    for t in range(num_points):
        im = np.sort(rng.choice(np.arange(1, num_images), L[t], replace=False))
        imgs.append(im)
        fts.append(rng.integers(0, nfeat[im]))
    track_offsets = np.zeros(num_points + 1, np.int64)
    track_offsets[1:] = np.cumsum(L)
    nc = int(rec.sum())
    aa = rng.normal(0, 0.6, (nc, 3))
    aa[:3][:nc] = [[0.0, 0.0, 0.0], [1e-9, -2e-9, 5e-10], [0.6 * (math.pi - 1e-7), -0.8 * (math.pi - 1e-7), 0.0]][:nc]
    refined_ext = np.column_stack([aa, rng.normal(0, 3, (nc, 3))])
    refined_intr = group_intr * (1 + rng.normal(0, 0.01, group_intr.shape))
    return {"cameras": cams, "reconstructed": rec, "intrinsic_group": image_group, "group_keys": group_keys,
            "group_intrinsics": group_intr, "feature_offsets": feature_offsets, "features": features,
            "track_keys": track_keys, "points": X, "track_offsets": track_offsets,
            "track_image": np.concatenate(imgs).astype(np.uint32),
            "track_feature": np.concatenate(fts).astype(np.uint32), "first_added": min(7, num_images - 1),
            "refined_extrinsics": refined_ext, "refined_intrinsics": refined_intr}


def engine_state_large(num_images=5000, num_points=2_000_000, seed=12, reconstructed_frac=0.8):
    """A full-size engine state (the large workload's 5,000 cameras and 2M
    points, track lengths 2..8, ~10M entries), built with numpy only: entries
    ascend by image inside a track, features are drawn per image."""
    rng = np.random.default_rng(seed)
    base = engine_state(num_images=num_images, num_points=8, seed=seed, reconstructed_frac=reconstructed_frac)
    L = rng.integers(2, 9, num_points)
    off = np.zeros(num_points + 1, np.int64)
    off[1:] = np.cumsum(L)
    ne = int(off[-1])
    start = rng.integers(1, num_images - 40, num_points)
    step = rng.integers(1, 5, ne)
    tr = np.repeat(np.arange(num_points), L)
    first_of = off[:-1][tr]
    step[np.arange(ne) == first_of] = 0
    cs = np.cumsum(step)
    img = start[tr] + cs - cs[first_of]
    nfeat = np.diff(base["feature_offsets"])
    nfeat[nfeat == 0] = 1
    fo = np.zeros(num_images + 1, np.int64)
    fo[1:] = np.cumsum(nfeat)
    st = dict(base)
    st.update(feature_offsets=fo, features=rng.uniform(0, 2000, (int(fo[-1]), 2)).astype(np.float32),
              points=rng.uniform(-2, 2, (num_points, 3)), track_offsets=off, track_image=img.astype(np.uint32),
              track_feature=(rng.random(ne) * nfeat[img]).astype(np.uint32), track_keys=np.arange(num_points))
    return st


def engine_state_sample(st, num_points):
    """The first `num_points` tracks of an engine state (same images,
    cameras and features)."""
    off = st["track_offsets"][:num_points + 1]
    out = dict(st)
    out.update(points=st["points"][:num_points], track_offsets=off, track_image=st["track_image"][:off[-1]],
               track_feature=st["track_feature"][:off[-1]], track_keys=st["track_keys"][:num_points])
    return out


def resection_scene(num_points=600, seed=13, outlier_frac=0.3, sigma=0.5, width=1920, height=1080):
    """2D-3D correspondences for a robust resection: one pinhole camera
    (f = 1000, principal point at the image centre) 8 units from a cloud of
    points, pixel noise, and a share of the 2D points replaced by uniform
    positions in the image (outliers)."""
    rng = np.random.default_rng(seed)
    center = np.array([[0.5, -0.3, -8.0]])
    R, t = _cameras_facing_origin(center)
    K = np.array([[1000.0, 0.0, width / 2], [0.0, 1000.0, height / 2], [0.0, 0.0, 1.0]])
    X = rng.uniform(-2.5, 2.5, (num_points, 3))
    p = X @ R[0].T + t[0]
    x = (p[:, :2] / p[:, 2:]) @ K[:2, :2].T + K[:2, 2]
    x += rng.normal(scale=sigma, size=x.shape)
    out = rng.random(num_points) < outlier_frac
    x[out] = rng.uniform([0, 0], [width, height], (out.sum(), 2))
    return {"x2d": x, "x3d": X, "K": K, "width": width, "height": height, "outlier": out.astype(np.uint8)}


def illconditioned_scene(num_cameras=24, num_points=3000, seed=17, baseline=0.01, radius=10.0, extent=2.0,
                         sigma=0.5, pair_frac=0.4, huber=4.0):
    """A scene whose point blocks are ill-conditioned: cameras come in twins
    `baseline` apart on a ring of radius 10, and a share of the points is
    seen by one twin pair only (rays meeting at ~0.06 degrees, so V's depth
    direction is ~1e6 times weaker than the others); the other points are
    seen by 3-8 cameras around the ring.  Per-camera radial K3 with the
    intrinsics held, Huber loss, cameras 0 and 1 held."""
    rng = np.random.default_rng(seed)
    half = num_cameras // 2
    theta = np.arange(half) * 2 * math.pi / half
    base = radius * np.stack([np.sin(theta), np.zeros_like(theta), np.cos(theta)], -1)
    tang = np.stack([np.cos(theta), np.zeros_like(theta), -np.sin(theta)], -1)
    centers = np.concatenate([base, base + baseline * tang])
    R, t = _cameras_facing_origin(centers)
    ext_true = np.concatenate([rotation_to_angle_axis(R), t], 1)
    intr = np.zeros((num_cameras, 6))
    intr[:, 0] = 1000.0
    intr[:, 1], intr[:, 2] = PP
    X_true = rng.uniform(-extent, extent, size=(num_points, 3))
    pairs = rng.random(num_points) < pair_frac
    cams, pts = [], []
    for p in range(num_points):
        if pairs[p]:
            k = int(rng.integers(0, half))
            c = np.array([k, half + k])
        else:
            c = np.sort(rng.choice(num_cameras, int(rng.integers(3, 9)), replace=False))
        cams.append(c)
        pts.append(np.full(len(c), p))
    cam = np.concatenate(cams)
    pt = np.concatenate(pts)
    intr_idx = cam.copy()
    obs, _, _ = _observe(rng, abi.RADIAL_K3, ext_true, intr, X_true, cam, intr_idx, pt, sigma)
    ext, X = _perturb(rng, ext_true.copy(), X_true, 0.002, 0.01, 0.02, fixed_cams=(0, 1))
    cam_const = np.zeros(num_cameras, np.uint8)
    cam_const[[0, 1]] = 1
    sc = _scene_dict(abi.RADIAL_K3, ext, intr, X, obs, cam, intr_idx, pt, camera_constant=cam_const,
                     intrinsic_constant=np.ones(num_cameras, np.uint8),
                     truth={"extrinsics": ext_true, "points": X_true, "intrinsics": intr.copy()},
                     name="illconditioned", seed=seed)
    sc["loss_scale"] = huber
    return sc
