"""The libs/sfm / libs/multiview adapter header compiles against the
reference's own headers (development container only: needs the reference
sources and the generated mvg/config.h stub of `make -C oracle ref`)."""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

import oracle

REF = oracle.reference_dir() or ""
GEN = os.path.join(ROOT, "oracle", "_ref", "gen")

SRC = r'''
#include "mvg/math/numeric.h"
#include "mvg/sfm/problem_data_container.h"
#include "mvg_gbba_adapter.h"
using namespace mvg::math;
void use_incremental(mvg::sfm::BA_Problem_data_camMotionAndIntrinsic<6, 6>& ba) {
  mvg::sfm::gpu::BundleAdjustmentOptions opt;
  opt.loss = GBBA_LOSS_HUBER; opt.loss_scale = 4.0; opt.intrinsic_fixed_mask = 0x3e;
  std::vector<uint8_t> cc(ba.num_cameras_, 0);
  gbba_summary s;
  mvg::sfm::gpu::SolveBundleAdjustment(ba, GBBA_RADIAL_K3, opt, cc, &s);
}
void use_unit_test(mvg::sfm::BAProblemData<7>& ba) {
  mvg::sfm::gpu::SolveBundleAdjustmentRtf(ba, mvg::sfm::gpu::BundleAdjustmentOptions(), nullptr);
}
void use_tri(const Mat34& P1, const Vec2& x1, const Mat34& P2, const Vec2& x2, const Mat2X& x,
             const std::vector<Mat34>& Ps) {
  Vec4 X;
  mvg::multiview::gpu::TriangulateDLT(P1, x1, P2, x2, &X);
  mvg::multiview::gpu::TriangulateNView(x, Ps, &X);
}
'''


@pytest.mark.skipif(not (os.path.isdir(REF) and os.path.isdir(GEN)), reason="reference sources not present")
def test_adapter_compiles_against_reference_headers():
    d = tempfile.mkdtemp()
    src = os.path.join(d, "use.cpp")
    open(src, "w").write(SRC)
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-w", "-I", GEN, "-I", os.path.join(REF, "3rdparty/eigen3"),
           "-I", os.path.join(REF, "libs/base/include"), "-I", os.path.join(REF, "libs/sfm/include"),
           "-I", os.path.join(ROOT, "3dreconstruction_gb300", "adapter"), src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
