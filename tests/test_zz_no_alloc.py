"""gbba_project_forward_noalloc: the forward projection for callers that
cannot allocate device memory (their memory belongs to another pool
allocator, or their loop may not pay an allocation's synchronisation).

It must give the same residuals and cost as the allocating entry point
gbba_project_forward -- residuals exactly (same arithmetic), the cost within
1e-12 relative (only the summation order differs) -- on calls in a row: each
problem twice, then a smaller problem, so that stale partial sums left in the
shared scratch by earlier calls must not leak into a result.  Kept in a file
of its own, collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def allocating_forward(handle, abi, sc, loss, a):
    hp = abi.HostProblem(sc)
    p = hp.struct()
    res = np.zeros((p.num_observations, 2))
    cost = np.zeros(1)
    handle.check(handle.lib.gbba_project_forward(handle.h, C.byref(p), loss, a, res.ctypes.data, cost.ctypes.data),
                 "gbba_project_forward")
    return res, cost[0]


def test_noalloc_forward_matches_allocating_entry(handle, abi, scenes):
    torch = pytest.importorskip("torch")
    lib = handle.lib
    stream = torch.cuda.current_stream()
    cases = [(scenes.medium_scene(num_cameras=40, num_points=6000, seed=91), abi.LOSS_HUBER, 4.0),
             (scenes.medium_scene(num_cameras=12, num_points=500, seed=92, model=abi.BROWN_T2), abi.LOSS_SQUARED, 1.0)]
    for sc, loss, a in cases:
        ref_res, ref_cost = allocating_forward(handle, abi, sc, loss, a)
        dp = abi.DeviceProblem(sc)
        p = dp.struct()
        free_delta = []
        for call in range(2):  # the same problem twice: the repeat may not take device memory
            res = torch.full((len(sc["observations"]), 2), -1.0, dtype=torch.float64, device="cuda")
            cost = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            st = lib.gbba_project_forward_noalloc(C.byref(p), loss, a, res.data_ptr(), cost.data_ptr(),
                                                  C.c_void_p(stream.cuda_stream))
            assert st == abi.SUCCESS
            torch.cuda.synchronize()
            free_delta.append(free_before - torch.cuda.mem_get_info()[0])
            np.testing.assert_array_equal(res.cpu().numpy(), ref_res)
            assert abs(cost.item() - ref_cost) <= 1e-12 * ref_cost
        # the first call of a camera model may load that kernel's code (lazy
        # module loading); a repeated call takes no device memory at all
        assert free_delta[1] == 0


def test_noalloc_rejects_oversized_and_host_problems(abi):
    import importlib
    lib = importlib.import_module("3dreconstruction_gb300").lib()
    p = abi.GbbaProblem()
    p.camera_model = abi.RADIAL_K3
    p.memory = abi.MEMORY_DEVICE
    p.num_observations = abi.NOALLOC_MAX_BLOCKS * abi.NOALLOC_OBS_PER_BLOCK + 1
    assert lib.gbba_project_forward_noalloc(C.byref(p), 0, 1.0, None, None, None) == abi.ERROR_TOO_LARGE
    p.memory = abi.MEMORY_HOST
    p.num_observations = 10
    assert lib.gbba_project_forward_noalloc(C.byref(p), 0, 1.0, None, None, None) == abi.ERROR_INVALID_ARGUMENT


def test_noalloc_out_of_range_index_gives_nan_then_recovers(handle, abi, scenes):
    """An observation whose point index is out of range gets NaN residuals and
    makes the cost NaN (the kernel checks every index before it reads); the
    next valid call clears the error slot and matches gbba_project_forward."""
    torch = pytest.importorskip("torch")
    lib = handle.lib
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    sc = scenes.medium_scene(num_cameras=10, num_points=300, seed=93)
    ref_res, ref_cost = allocating_forward(handle, abi, sc, abi.LOSS_HUBER, 4.0)
    bad = dict(sc)
    bad["point_index"] = sc["point_index"].copy()
    bad["point_index"][7] = len(sc["points"]) + 5
    no = len(sc["observations"])
    for scene, expect_nan in ((bad, True), (sc, False)):
        dp = abi.DeviceProblem(scene)
        p = dp.struct()
        res = torch.full((no, 2), -1.0, dtype=torch.float64, device="cuda")
        cost = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        st = lib.gbba_project_forward_noalloc(C.byref(p), abi.LOSS_HUBER, 4.0, res.data_ptr(), cost.data_ptr(), stream)
        assert st == abi.SUCCESS
        torch.cuda.synchronize()
        r = res.cpu().numpy()
        if expect_nan:
            assert np.isnan(r[7]).all() and np.isnan(cost.item())
            ok = np.ones(no, bool)
            ok[7] = False
            np.testing.assert_array_equal(r[ok], ref_res[ok])
        else:
            np.testing.assert_array_equal(r, ref_res)
            assert np.isfinite(cost.item()) and abs(cost.item() - ref_cost) <= 1e-12 * ref_cost
