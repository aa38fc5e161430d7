"""ls_matvec_host with page-locked host buffers: the matvec reads x from and
writes y to host memory directly (no separate copies). Its result must be
bit for bit the one of the copy path (pageable numpy buffers) and of the
device entry point, for the native and the double-float kernels."""
import ctypes

import numpy as np
import pytest

from conftest import CFG_C1, full_cfg

pytestmark = pytest.mark.gpu


def test_pinned_host_buffers_give_the_copy_path_result(ls):
    torch = pytest.importorskip("torch")
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N)
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.zeros_like(xh).pin_memory()
    dp = ctypes.POINTER(ctypes.c_double)
    for kernels in (ls.LS_F64_NATIVE, ls.LS_F64_DOUBLE_FLOAT):
        op.set_f64_kernels(kernels)
        y_copy = op.matvec(x)  # pageable buffers: copy path
        for _ in range(2):  # twice: the buffers are reused as a caller would
            rc = ls.lib().ls_matvec_host(op._h, ctypes.cast(xh.data_ptr(), dp), ctypes.cast(yh.data_ptr(), dp))
            assert rc == ls.LS_OK
            assert np.array_equal(yh.numpy(), y_copy)
        xd = torch.from_numpy(x).cuda()
        yd = torch.empty_like(xd)
        op.matvec_device(xd.data_ptr(), yd.data_ptr(), 0)
        torch.cuda.synchronize()
        assert np.array_equal(yd.cpu().numpy(), y_copy)
    op.close()


def test_graph_of_the_host_buffer_matvec_follows_buffers_and_settings(ls):
    """The page-locked path runs the matvec as a captured CUDA graph, keyed by
    the buffers, the kernel family and the launch schedule: new buffers,
    another kernel family and another near-field schedule each give a new
    graph whose result equals the copy path's, bit for bit."""
    torch = pytest.importorskip("torch")
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    rng = np.random.default_rng(5)
    dp = ctypes.POINTER(ctypes.c_double)
    was = ls.get_near_overlap()
    try:
        for trial in range(2):  # a second pair of buffers forces a recapture
            x = rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N)
            xh = torch.from_numpy(x).pin_memory()
            yh = torch.zeros_like(xh).pin_memory()
            for kernels in (ls.LS_F64_NATIVE, ls.LS_F64_DOUBLE_FLOAT, ls.LS_F64_NATIVE):
                op.set_f64_kernels(kernels)
                for overlap in (True, False, True):
                    ls.set_near_overlap(overlap)
                    y_copy = op.matvec(x)
                    for _ in range(2):  # the second call replays the graph
                        rc = ls.lib().ls_matvec_host(op._h, ctypes.cast(xh.data_ptr(), dp),
                                                     ctypes.cast(yh.data_ptr(), dp))
                        assert rc == 0, ls.lib().ls_last_error()
                        assert np.array_equal(yh.numpy(), y_copy), (trial, kernels, overlap)
    finally:
        ls.set_near_overlap(was)
        op.set_f64_kernels(ls.LS_F64_NATIVE)
    op.close()
