"""ctypes mirror of include/gbba.h and include/gbtri.h.

The structures here are byte-for-byte the C structs of the boundary; the
helpers build a `gbba_problem` from numpy arrays (host memory) or from CUDA
tensors (device memory, via their data pointers).
"""
import ctypes as C

import numpy as np

# gbba_status
SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_CUDA = 2
ERROR_OUT_OF_MEMORY = 3
ERROR_NUMERICAL = 4
ERROR_NOT_SUPPORTED = 5
ERROR_TOO_LARGE = 6
ERROR_NO_DEVICE = 7
ERROR_TIMEOUT = 8

# gbba_camera_model
PINHOLE_F = 0
RADIAL_K3 = 1
BROWN_T2 = 2
MODEL_K = {PINHOLE_F: 1, RADIAL_K3: 6, BROWN_T2: 8}

LOSS_SQUARED = 0
LOSS_HUBER = 1

SOLVER_AUTO = 0
SOLVER_DENSE_SCHUR = 1
SOLVER_ITERATIVE_SCHUR = 2
SCHUR_BUILD_AUTO = 0
SCHUR_BUILD_POINT_ATOMIC = 1

PRECISION_FP64 = 0
PRECISION_MIXED = 1

MEMORY_HOST = 0
MEMORY_DEVICE = 1

CONVERGENCE = 0
NO_CONVERGENCE = 1
FAILURE = 2

NOALLOC_MAX_BLOCKS = 16384
NOALLOC_OBS_PER_BLOCK = 2048

# gbtri_method
TRI_NVIEW = 0
TRI_NVIEW_ALGEBRAIC = 1
TRI_ITERATIVE = 2
TRACK_OK = 0
TRACK_DEGENERATE = 1
TRACK_BEHIND_CAMERA = 2


class GbbaProblem(C.Structure):
    _fields_ = [
        ("camera_model", C.c_int32),
        ("memory", C.c_int32),
        ("num_cameras", C.c_int64),
        ("num_intrinsics", C.c_int64),
        ("num_points", C.c_int64),
        ("num_observations", C.c_int64),
        ("extrinsics", C.c_void_p),
        ("intrinsics", C.c_void_p),
        ("points", C.c_void_p),
        ("observations", C.c_void_p),
        ("camera_index", C.c_void_p),
        ("intrinsic_index", C.c_void_p),
        ("point_index", C.c_void_p),
        ("camera_constant", C.c_void_p),
        ("intrinsic_constant", C.c_void_p),
        ("extrinsic_fixed_mask", C.c_uint32),
        ("intrinsic_fixed_mask", C.c_uint32),
    ]


class GbbaOptions(C.Structure):
    _fields_ = [
        ("max_num_iterations", C.c_int32),
        ("max_num_consecutive_invalid_steps", C.c_int32),
        ("function_tolerance", C.c_double),
        ("gradient_tolerance", C.c_double),
        ("parameter_tolerance", C.c_double),
        ("initial_trust_region_radius", C.c_double),
        ("max_trust_region_radius", C.c_double),
        ("min_trust_region_radius", C.c_double),
        ("min_relative_decrease", C.c_double),
        ("min_lm_diagonal", C.c_double),
        ("max_lm_diagonal", C.c_double),
        ("jacobi_scaling", C.c_int32),
        ("loss_type", C.c_int32),
        ("loss_scale", C.c_double),
        ("linear_solver", C.c_int32),
        ("precision", C.c_int32),
        ("max_linear_solver_iterations", C.c_int32),
        ("dense_schur_max_size", C.c_int32),
        ("eta", C.c_double),
        ("refinement_interval", C.c_int32),
        ("use_cuda_graphs", C.c_int32),
        ("stream", C.c_void_p),
        ("fp64_polish_iterations", C.c_int32),
        ("schur_build", C.c_int32),
        ("trace_cost", C.c_void_p),
        ("trace_time_s", C.c_void_p),
        ("trace_capacity", C.c_int32),
        ("mixed_flags", C.c_uint32),
    ]


class GbbaSummary(C.Structure):
    _fields_ = [
        ("initial_cost", C.c_double),
        ("final_cost", C.c_double),
        ("num_iterations", C.c_int32),
        ("num_successful_steps", C.c_int32),
        ("num_unsuccessful_steps", C.c_int32),
        ("termination_type", C.c_int32),
        ("usable", C.c_int32),
        ("linear_solver_iterations", C.c_int32),
        ("reduced_system_size", C.c_int64),
        ("total_time_s", C.c_double),
        ("jacobian_time_s", C.c_double),
        ("linear_solver_time_s", C.c_double),
        ("residual_time_s", C.c_double),
        ("schur_kernel_time_s", C.c_double),
        ("schur_kernel_launches", C.c_int32),
        ("factor_launches", C.c_int32),
        ("factor_time_s", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


TUNE_MAX_CANDIDATES = 4


class GbbaTuning(C.Structure):
    _fields_ = [
        ("pair_chunk", C.c_int32),
        ("num_candidates", C.c_int32),
        ("candidates", C.c_int32 * TUNE_MAX_CANDIDATES),
        ("schur_time_s", C.c_double * TUNE_MAX_CANDIDATES),
        ("factor_tensor", C.c_int32),
        ("camera_warps", C.c_int32),
        ("factor_time_s", C.c_double * 2),
        ("pcg_time_s", C.c_double * 3),
    ]


class GbsfmCamera(C.Structure):
    """gbsfm_camera: rotation (row-major), translation, f, ppx, ppy, k1, k2, k3;
    the same 18 doubles as a row of scenes.brown_cameras()."""
    _fields_ = [("R", C.c_double * 9), ("t", C.c_double * 3), ("f", C.c_double), ("ppx", C.c_double),
                ("ppy", C.c_double), ("k1", C.c_double), ("k2", C.c_double), ("k3", C.c_double)]


class GbsfmResidualStats(C.Structure):
    _fields_ = [("count", C.c_int64), ("min", C.c_double), ("max", C.c_double), ("mean", C.c_double),
                ("median", C.c_double), ("hist", C.c_int64 * 10), ("underflow", C.c_int64), ("overflow", C.c_int64)]


LOCK_AS_REFERENCE, LOCK_FIRST_ADDED, LOCK_NONE = 0, 1, 2
MIXED_KAHAN_SCHUR, MIXED_FP64_POINT_INVERSE = 1, 2


class GbsfmAcransacParams(C.Structure):
    _fields_ = [("sample_size", C.c_int32), ("max_models", C.c_int32), ("logalpha0", C.c_double),
                ("mult_error", C.c_double), ("max_threshold", C.c_double)]


class GbsfmEngineState(C.Structure):
    """gbsfm_engine_state: the incremental engine's maps as dense arrays."""
    _fields_ = [("num_images", C.c_int64), ("cameras", C.c_void_p), ("reconstructed", C.c_void_p),
                ("intrinsic_group", C.c_void_p), ("num_intrinsic_groups", C.c_int64),
                ("group_intrinsics", C.c_void_p), ("num_features", C.c_int64), ("feature_offsets", C.c_void_p),
                ("features", C.c_void_p), ("num_points", C.c_int64), ("points", C.c_void_p),
                ("num_entries", C.c_int64), ("track_offsets", C.c_void_p), ("track_image", C.c_void_p),
                ("track_feature", C.c_void_p)]


class GbsfmBaArrays(C.Structure):
    """gbsfm_ba_arrays: outputs of gbsfm_pack_ba."""
    _fields_ = [("extrinsics", C.c_void_p), ("intrinsics", C.c_void_p), ("points", C.c_void_p),
                ("observations", C.c_void_p), ("camera_index", C.c_void_p), ("intrinsic_index", C.c_void_p),
                ("point_index", C.c_void_p), ("camera_constant", C.c_void_p), ("camera_image", C.c_void_p),
                ("num_cameras", C.c_int64), ("num_observations", C.c_int64), ("measurements", C.c_int64),
                ("locked_camera", C.c_int64)]


def default_options(**kw):
    """ceres::Solver::Options defaults (include/ceres/solver.h:81-129)."""
    o = GbbaOptions()
    o.max_num_iterations = 50
    o.max_num_consecutive_invalid_steps = 5
    o.function_tolerance = 1e-6
    o.gradient_tolerance = 1e-10
    o.parameter_tolerance = 1e-8
    o.initial_trust_region_radius = 1e4
    o.max_trust_region_radius = 1e16
    o.min_trust_region_radius = 1e-32
    o.min_relative_decrease = 1e-3
    o.min_lm_diagonal = 1e-6
    o.max_lm_diagonal = 1e32
    o.jacobi_scaling = 1
    o.loss_type = LOSS_SQUARED
    o.loss_scale = 1.0
    o.linear_solver = SOLVER_AUTO
    o.precision = PRECISION_FP64
    o.max_linear_solver_iterations = 500
    o.dense_schur_max_size = 16384
    o.eta = 0.1
    o.refinement_interval = 10
    o.use_cuda_graphs = 1
    o.stream = None
    o.fp64_polish_iterations = 10
    o.schur_build = 0
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


class HostProblem:
    """Owns numpy arrays of a BA problem and exposes a GbbaProblem over them.

    Parameter arrays are refined in place by a solve."""

    FIELDS = ("extrinsics", "intrinsics", "points", "observations", "camera_index",
              "intrinsic_index", "point_index", "camera_constant", "intrinsic_constant")

    def __init__(self, scene, copy=True):
        self.model = int(scene["model"])
        conv = {
            "extrinsics": np.float64, "intrinsics": np.float64, "points": np.float64,
            "observations": np.float64, "camera_index": np.uint32, "intrinsic_index": np.uint32,
            "point_index": np.uint32, "camera_constant": np.uint8, "intrinsic_constant": np.uint8,
        }
        for f in self.FIELDS:
            v = scene.get(f)
            if v is None:
                setattr(self, f, None)
                continue
            a = np.ascontiguousarray(np.asarray(v, dtype=conv[f]))
            setattr(self, f, a.copy() if copy else a)
        self.extrinsic_fixed_mask = int(scene.get("extrinsic_fixed_mask", 0))
        self.intrinsic_fixed_mask = int(scene.get("intrinsic_fixed_mask", 0))

    def struct(self):
        p = GbbaProblem()
        p.camera_model = self.model
        p.memory = MEMORY_HOST
        p.num_cameras = self.extrinsics.size // 6
        p.num_intrinsics = self.intrinsics.size // MODEL_K[self.model]
        p.num_points = self.points.size // 3
        p.num_observations = self.observations.size // 2
        for f in self.FIELDS:
            setattr(p, f, _ptr(getattr(self, f)))
        p.extrinsic_fixed_mask = self.extrinsic_fixed_mask
        p.intrinsic_fixed_mask = self.intrinsic_fixed_mask
        return p

    def params(self):
        return {"extrinsics": self.extrinsics.copy(), "intrinsics": self.intrinsics.copy(),
                "points": self.points.copy()}


class DeviceProblem:
    """The same problem resident in device memory (torch CUDA tensors)."""

    def __init__(self, scene, device="cuda:0"):
        import torch
        self.model = int(scene["model"])
        conv = {
            "extrinsics": torch.float64, "intrinsics": torch.float64, "points": torch.float64,
            "observations": torch.float64, "camera_index": torch.int32, "intrinsic_index": torch.int32,
            "point_index": torch.int32, "camera_constant": torch.uint8, "intrinsic_constant": torch.uint8,
        }
        for f in HostProblem.FIELDS:
            v = scene.get(f)
            if v is None:
                setattr(self, f, None)
                continue
            a = np.ascontiguousarray(np.asarray(v))
            if a.dtype == np.uint32:
                a = a.view(np.int32)
            setattr(self, f, torch.from_numpy(a.copy()).to(device=device, dtype=conv[f]).contiguous())
        self.extrinsic_fixed_mask = int(scene.get("extrinsic_fixed_mask", 0))
        self.intrinsic_fixed_mask = int(scene.get("intrinsic_fixed_mask", 0))

    def struct(self):
        p = GbbaProblem()
        p.camera_model = self.model
        p.memory = MEMORY_DEVICE
        p.num_cameras = self.extrinsics.numel() // 6
        p.num_intrinsics = self.intrinsics.numel() // MODEL_K[self.model]
        p.num_points = self.points.numel() // 3
        p.num_observations = self.observations.numel() // 2
        for f in HostProblem.FIELDS:
            setattr(p, f, _ptr(getattr(self, f)))
        p.extrinsic_fixed_mask = self.extrinsic_fixed_mask
        p.intrinsic_fixed_mask = self.intrinsic_fixed_mask
        return p

    def params(self):
        return {"extrinsics": self.extrinsics.cpu().numpy(), "intrinsics": self.intrinsics.cpu().numpy(),
                "points": self.points.cpu().numpy()}


class EnginePack:
    """An engine state (the dict of scenes.engine_state()) and the output
    arrays of gbsfm_pack_ba, on the host (numpy) or on a device (torch), with
    the structs that point at them."""

    STATE = {"cameras": np.float64, "reconstructed": np.uint8, "intrinsic_group": np.uint32,
             "group_intrinsics": np.float64, "feature_offsets": np.int64, "features": np.float32,
             "points": np.float64, "track_offsets": np.int64, "track_image": np.uint32, "track_feature": np.uint32}

    def __init__(self, state, device=None):
        self.device = device
        self.ni = len(state["reconstructed"])
        self.ng = len(np.asarray(state["group_intrinsics"]).reshape(-1, 6))
        self.nf = len(np.asarray(state["features"]).reshape(-1, 2))
        self.nt = len(state["track_offsets"]) - 1
        self.ne = len(state["track_image"])
        self.arrays = {k: self._put(np.ascontiguousarray(np.asarray(state[k], t))) for k, t in self.STATE.items()}
        shapes = {"extrinsics": (6 * self.ni, np.float64), "intrinsics": (6 * self.ng, np.float64),
                  "points": (3 * self.nt, np.float64), "observations": (2 * self.ne, np.float64),
                  "camera_index": (self.ne, np.uint32), "intrinsic_index": (self.ne, np.uint32),
                  "point_index": (self.ne, np.uint32), "camera_constant": (self.ni, np.uint8),
                  "camera_image": (self.ni, np.uint32)}
        self.out = {k: self._put(np.zeros(max(n, 1), t)) for k, (n, t) in shapes.items()}
        self.memory = MEMORY_HOST if device is None else MEMORY_DEVICE

    def _put(self, a):
        if self.device is None:
            return a
        import torch
        if a.dtype == np.uint32:
            a = a.view(np.int32)
        return torch.from_numpy(a.copy()).to(self.device)

    def state_struct(self):
        s = GbsfmEngineState()
        a = self.arrays
        s.num_images, s.num_intrinsic_groups, s.num_features = self.ni, self.ng, self.nf
        s.num_points, s.num_entries = self.nt, self.ne
        for k in ("cameras", "reconstructed", "intrinsic_group", "group_intrinsics", "feature_offsets", "features",
                  "points", "track_offsets", "track_image", "track_feature"):
            setattr(s, k, _ptr(a[k]))
        return s

    def out_struct(self):
        o = GbsfmBaArrays()
        for k, v in self.out.items():
            setattr(o, k, _ptr(v))
        return o

    def pack(self, lib, h, first_added, lock=LOCK_AS_REFERENCE):
        """Runs gbsfm_pack_ba; returns (status, GbsfmBaArrays)."""
        s, o = self.state_struct(), self.out_struct()
        st = lib.gbsfm_pack_ba(h, C.byref(s), int(first_added), int(lock), C.byref(o), self.memory)
        return st, o

    def result(self, o):
        """The packed problem as numpy arrays, cut to the counts of `o`."""
        nc, no = o.num_cameras, o.num_observations
        get = {}
        for k, v in self.out.items():
            a = v if self.device is None else v.cpu().numpy()
            if k in ("camera_index", "intrinsic_index", "point_index", "camera_image"):
                a = a.view(np.uint32)
            get[k] = a
        return {"extrinsics": get["extrinsics"][:6 * nc].reshape(-1, 6), "intrinsics": get["intrinsics"][:6 * self.ng],
                "points": get["points"][:3 * self.nt], "observations": get["observations"][:2 * no].reshape(-1, 2),
                "camera_index": get["camera_index"][:no], "intrinsic_index": get["intrinsic_index"][:no],
                "point_index": get["point_index"][:no], "camera_constant": get["camera_constant"][:nc],
                "camera_image": get["camera_image"][:nc], "num_cameras": nc, "num_observations": no,
                "measurements": o.measurements, "locked_camera": o.locked_camera}


def declare_gbba(lib):
    """Attach argument / return types to the C-ABI symbols of libgbba."""
    P = C.POINTER
    vp = C.c_void_p
    lib.gbba_create.argtypes = [C.c_int, P(vp)]
    lib.gbba_create.restype = C.c_int
    lib.gbba_destroy.argtypes = [vp]
    lib.gbba_destroy.restype = None
    lib.gbba_default_options.argtypes = [P(GbbaOptions)]
    lib.gbba_default_options.restype = None
    lib.gbba_status_string.argtypes = [C.c_int]
    lib.gbba_status_string.restype = C.c_char_p
    lib.gbba_abi_version.argtypes = []
    lib.gbba_abi_version.restype = C.c_int
    lib.gbba_launch_count.argtypes = [vp]
    lib.gbba_launch_count.restype = C.c_int64
    lib.gbba_solve.argtypes = [vp, P(GbbaProblem), P(GbbaOptions), P(GbbaSummary)]
    lib.gbba_solve.restype = C.c_int
    lib.gbba_solve_batched.argtypes = [vp, P(GbbaProblem), C.c_int32, P(GbbaOptions), P(GbbaSummary)]
    lib.gbba_solve_batched.restype = C.c_int
    lib.gbba_autotune.argtypes = [vp, P(GbbaProblem), P(GbbaOptions), C.c_int32, P(GbbaTuning)]
    lib.gbba_autotune.restype = C.c_int
    lib.gbba_project_forward.argtypes = [vp, P(GbbaProblem), C.c_int32, C.c_double, vp, vp]
    lib.gbba_project_forward.restype = C.c_int
    lib.gbba_project_backward.argtypes = [vp, P(GbbaProblem), C.c_int32, C.c_double, vp, vp, vp, vp]
    lib.gbba_project_backward.restype = C.c_int
    lib.gbba_project_backward_mixed.argtypes = [vp, P(GbbaProblem), C.c_int32, C.c_double, vp, vp, vp, vp]
    lib.gbba_project_backward_mixed.restype = C.c_int
    lib.gbba_project_forward_noalloc.argtypes = [P(GbbaProblem), C.c_int32, C.c_double, vp, vp, vp]
    lib.gbba_project_forward_noalloc.restype = C.c_int
    lib.gbsfm_triangulate_pair.argtypes = [vp, vp, vp, C.c_int64, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                                           vp, vp, vp, vp, C.c_int32]
    lib.gbsfm_triangulate_pair.restype = C.c_int
    lib.gbsfm_reject_tracks.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, vp, vp, vp, C.c_double, C.c_double, vp, vp,
                                        vp, vp, C.c_int32]
    lib.gbsfm_reject_tracks.restype = C.c_int
    lib.gbsfm_residual_histogram.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, vp, vp, vp, P(GbsfmResidualStats),
                                             C.c_int32]
    lib.gbsfm_residual_histogram.restype = C.c_int
    lib.gbsfm_pack_ba.argtypes = [vp, P(GbsfmEngineState), C.c_int64, C.c_int32, P(GbsfmBaArrays), C.c_int32]
    lib.gbsfm_pack_ba.restype = C.c_int
    lib.gbsfm_unpack_ba.argtypes = [vp, C.c_int64, vp, vp, vp, C.c_int64, vp, C.c_int64, vp, C.c_int32]
    lib.gbsfm_unpack_ba.restype = C.c_int
    lib.gbsfm_acransac_score.argtypes = [vp, P(GbsfmAcransacParams), C.c_int64, vp, vp, C.c_int64, vp, vp, vp, vp,
                                         vp, C.c_int32]
    lib.gbsfm_acransac_score.restype = C.c_int
    lib.gbba_last_kernel_time.argtypes = [vp, vp]
    lib.gbba_last_kernel_time.restype = C.c_int
    lib.gbtri_dlt2_batched.argtypes = [vp, C.c_int64, vp, vp, C.c_int64, vp, vp, vp, vp, C.c_int32]
    lib.gbtri_dlt2_batched.restype = C.c_int
    lib.gbtri_nview_batched.argtypes = [vp, C.c_int32, vp, C.c_int64, vp, vp, vp, C.c_int64, vp, vp, C.c_int32]
    lib.gbtri_nview_batched.restype = C.c_int
    lib.gbtri_nview_batched_f32.argtypes = [vp, C.c_int32, vp, C.c_int64, vp, vp, vp, C.c_int64, C.c_int32, vp, vp, vp,
                                            C.c_int32]
    lib.gbtri_nview_batched_f32.restype = C.c_int
    lib.gbtri_refine_gn.argtypes = [vp, vp, C.c_int64, vp, vp, vp, C.c_int64, C.c_int32, vp, C.c_int32]
    lib.gbtri_refine_gn.restype = C.c_int
    return lib


# Every symbol the C-ABI headers declare (checked by the CPU tests).
EXPORTED_SYMBOLS = (
    "gbba_create", "gbba_destroy", "gbba_default_options", "gbba_status_string",
    "gbba_abi_version", "gbba_launch_count", "gbba_last_kernel_time", "gbba_solve", "gbba_solve_batched", "gbba_autotune",
    "gbba_project_forward", "gbba_project_backward", "gbba_project_backward_mixed", "gbba_project_forward_noalloc",
    "gbtri_dlt2_batched", "gbtri_nview_batched", "gbtri_nview_batched_f32", "gbtri_refine_gn",
    "gbsfm_triangulate_pair", "gbsfm_reject_tracks", "gbsfm_residual_histogram", "gbsfm_pack_ba",
    "gbsfm_unpack_ba", "gbsfm_acransac_score",
)
