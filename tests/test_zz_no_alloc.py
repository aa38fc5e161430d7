"""ls_matvec_noalloc: the matvec with its scratch in the library's static
device array, for callers that cannot allocate device memory while they run
(e.g. a solver embedded in a framework whose caching allocator owns the
device heap). Its output must match the regular ls_matvec on the same
inputs, on consecutive calls that reuse the shared array.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test.
"""
import numpy as np
import pytest

from conftest import CFG_C1, full_cfg

pytestmark = pytest.mark.gpu

TOL_PARITY = 1e-10  # the tolerance of the matvec parity tests


def test_noalloc_matches_regular_matvec_on_two_calls(ls):
    torch = pytest.importorskip("torch")
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    rng = np.random.default_rng(2024)
    for call in range(2):
        x = rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N)
        xt = torch.from_numpy(x).to("cuda:0")
        y_regular = torch.empty_like(xt)
        y_static = torch.full_like(xt, float("nan"))
        op.matvec_device(xt.data_ptr(), y_regular.data_ptr(), 0)
        op.matvec_device_noalloc(xt.data_ptr(), y_static.data_ptr(), 0)
        torch.cuda.synchronize()
        a, b = y_static.cpu().numpy(), y_regular.cpu().numpy()
        assert np.isfinite(a).all(), f"call {call}: non-finite output"
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= TOL_PARITY, f"call {call}"
    op.close()
