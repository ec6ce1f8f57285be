"""GB300-native bundle adjustment and triangulation (drop-in for the ceres /
Eigen path of yueying/3DReconstruction's libs/sfm and libs/multiview).

The compute lives in `libgbba.so` (CUDA for sm_103a behind the C ABI of
include/gbba.h and include/gbtri.h); this package only loads it and mirrors
its structures for Python callers (tests, benchmark).
"""
import ctypes
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbba.so")
_lib = None


def lib():
    """The loaded C-ABI library.  Raises if it has not been built: there is
    no fallback implementation."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        _lib = abi.declare_gbba(ctypes.CDLL(LIB_PATH))
    return _lib


class Handle:
    """Owns a gbba_handle (one CUDA stream + reusable workspace) on a device."""

    def __init__(self, device=0):
        self.lib = lib()
        h = ctypes.c_void_p()
        st = self.lib.gbba_create(device, ctypes.byref(h))
        if st != abi.SUCCESS:
            raise RuntimeError(f"gbba_create failed: {self.lib.gbba_status_string(st).decode()}")
        self.h = h

    def close(self):
        if self.h:
            self.lib.gbba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st, what):
        if st != abi.SUCCESS:
            raise RuntimeError(f"{what} failed: {self.lib.gbba_status_string(st).decode()} ({st})")

    def launches(self):
        return int(self.lib.gbba_launch_count(self.h))

    def solve(self, problem, options):
        """problem: abi.HostProblem / abi.DeviceProblem; refined in place."""
        s = abi.GbbaSummary()
        p = problem.struct()
        st = self.lib.gbba_solve(self.h, ctypes.byref(p), ctypes.byref(options), ctypes.byref(s))
        self.check(st, "gbba_solve")
        return s
