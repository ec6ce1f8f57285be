"""The per-track triangulation math of the CUDA kernels
(3dreconstruction_gb300/csrc/gbtri_track.cuh) compiled as host code and run
on the CPU against the reference's outputs: TriangulateNView,
TriangulateNViewAlgebraic and Triangulation::compute(3)
(libs/multiview/src/triangulation_nview.cpp:8-121) from ref_harness, on the
unit-test ring scenes, noisy tracks, tracks of the batched workload's
distributions and tracks of 33-150 views.

Tolerances: FP64 1e-9 relative (homogeneous vectors up to sign).  FP32, on
Euclidean points of the [-3,3]^3 scene from inputs that the reference also
saw rounded to FP32: median 1e-5, 99th percentile 5e-5, worst 5e-3 (short
tracks with near-parallel rays are the worst conditioned)."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, load_golden

CSRC = os.path.join(ROOT, "3dreconstruction_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "host", "tri_track_check.cu")
CASES = ["tri_ring_2x12.npz", "tri_ring_5x6.npz", "tri_noisy.npz", "tri_tracks_f32.npz", "tri_long.npz"]


@pytest.fixture(scope="module")
def host_exe():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "tri_track_check")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-O2", "-x", "cu", "-I", CSRC, SRC, "-o", exe],
                   check=True, capture_output=True)
    return exe


def run_host(exe, P, off, cam, xy):
    nt = len(off) - 1
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 12)
    d = tempfile.mkdtemp()
    fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(fin, "wb") as f:
        np.array([nt, len(P)], np.int64).tofile(f)
        P.tofile(f)
        np.asarray(off, np.int64).tofile(f)
        np.asarray(cam, np.uint32).tofile(f)
        np.asarray(xy, np.float64).reshape(-1, 2).tofile(f)
    subprocess.run([exe, fin, fout], check=True)
    o = np.fromfile(fout, np.float64)
    out, k = [], 0
    for w in (4, 4, 3, 4, 4, 3):
        out.append(o[k:k + w * nt].reshape(nt, w))
        k += w * nt
    return out


def sign_aligned_error(a, b):
    s = np.sign((a * b).sum(1))[:, None]
    return np.abs(a * s - b).max(1) / np.maximum(1.0, np.abs(b).max(1))


@pytest.mark.parametrize("case", CASES)
def test_track_math_matches_reference(case, host_exe):
    g = load_golden(case)
    nt = len(g["track_offsets"]) - 1
    nv, al, it, nv32, al32, it32 = run_host(host_exe, g["P"].astype(np.float64), g["track_offsets"],
                                            g["camera_index"], g["xy"].astype(np.float64))
    assert sign_aligned_error(nv, g["nview_h"].reshape(nt, 4)).max() < 1e-9
    assert sign_aligned_error(al, g["algebraic_h"].reshape(nt, 4)).max() < 1e-9
    np.testing.assert_allclose(it, g["iterative_e"].reshape(nt, 3), rtol=1e-9, atol=1e-9)
    ref_nv = g["nview_h"].reshape(nt, 4)
    ref_al = g["algebraic_h"].reshape(nt, 4)
    for got, ref in ((nv32[:, :3] / nv32[:, 3:], ref_nv[:, :3] / ref_nv[:, 3:]),
                     (al32[:, :3] / al32[:, 3:], ref_al[:, :3] / ref_al[:, 3:]),
                     (it32, g["iterative_e"].reshape(nt, 3))):
        err = np.abs(got - ref).max(1) / np.maximum(1.0, np.abs(ref).max(1))
        assert np.median(err) < 1e-5 and np.quantile(err, 0.99) < 5e-5 and err.max() < 5e-3, \
            (np.median(err), np.quantile(err, 0.99), err.max())
