"""ls_matvec_noalloc: the matvec with its scratch in the library's static
device array, for callers that cannot allocate device memory while they run
(e.g. a solver embedded in a framework whose caching allocator owns the
device heap). Its output must match the regular ls_matvec and the CPU
oracle on the same inputs, on consecutive calls that reuse the shared array.
It always runs the native FP64 kernels, also when the double-float kernels
are selected for the other FP64 entry points.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test.
"""
import numpy as np
import pytest

from conftest import CFG_C1, CFG_HFR, full_cfg

pytestmark = pytest.mark.gpu

TOL_PARITY = 1e-10  # the tolerance of the matvec parity tests


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("base", [CFG_C1, CFG_HFR])
def test_noalloc_matches_regular_matvec_and_oracle_on_two_calls(ls, ora, base):
    torch = pytest.importorskip("torch")
    cfg = full_cfg(base)
    op = ls.Operator(cfg, device=0)
    ref = ora.Oracle(cfg.as_dict())
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
        assert _rel(a, b) <= TOL_PARITY, f"call {call}"
        assert _rel(a, ref.matvec(x)) <= TOL_PARITY, f"call {call}: against the oracle"
    op.close()


def test_noalloc_runs_native_kernels_when_double_float_is_selected(ls):
    torch = pytest.importorskip("torch")
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    x = np.random.default_rng(5).uniform(-1, 1, op.N) + 1j * np.random.default_rng(6).uniform(-1, 1, op.N)
    xt = torch.from_numpy(x).to("cuda:0")
    y_before = torch.empty_like(xt)
    op.matvec_device_noalloc(xt.data_ptr(), y_before.data_ptr(), 0)
    op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    y_after = torch.empty_like(xt)
    op.matvec_device_noalloc(xt.data_ptr(), y_after.data_ptr(), 0)
    torch.cuda.synchronize()
    # Same kernels, same inputs: bitwise identical.
    assert torch.equal(y_before, y_after)
    op.close()
