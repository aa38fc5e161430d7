"""The FP32 operator on the tensor cores for 64 right-hand sides at once
(csrc/batched_tc.cu: tcgen05 MMAs, TF32 inputs in three products, FP32
accumulation in tensor memory), against the single-vector FP32 operator on
CUDA cores and the FP64 operator; and the batched mixed-precision solver
with 64-wide blocks against the 8-wide CUDA-core one."""
import numpy as np
import pytest

from conftest import CFG_C1, CFG_HFR, CFG_L3_K10, CFG_L5_BUMPS, full_cfg

pytestmark = pytest.mark.gpu


def _cols(n, k, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.uniform(-1, 1, (n, k)) + 1j * rng.uniform(-1, 1, (n, k)))


def _f32_single(ls, op, X):
    torch = pytest.importorskip("torch")
    out = np.empty_like(X)
    for j in range(X.shape[1]):
        xt = torch.from_numpy(np.ascontiguousarray(X[:, j])).cuda()
        yt = torch.empty_like(xt)
        op.matvec_device(xt.data_ptr(), yt.data_ptr(), 0, precision=ls.LS_PREC_F32)
        torch.cuda.synchronize()
        out[:, j] = yt.cpu().numpy()
    return out


@pytest.mark.parametrize("base,over,k", [(CFG_C1, {}, 64), (CFG_HFR, {}, 70), (CFG_L5_BUMPS, {}, 64),
                                         (CFG_L3_K10, {"nChebNodes": 8}, 64), (CFG_C1, {"findPhi": 0}, 64)])
def test_tensor_core_apply_matches_fp32_and_fp64_operators(ls, base, over, k):
    op = ls.Operator(full_cfg(base, **over), device=0)
    op.enable_f32()
    X = _cols(op.N, k, 3)
    Y = op.matvec_f32_many(X)
    Y32 = _f32_single(ls, op, X)
    e_tc, e_32 = [], []
    for j in range(k):
        y64 = op.matvec(np.ascontiguousarray(X[:, j]))
        e_tc.append(np.linalg.norm(Y[:, j] - y64) / np.linalg.norm(y64))
        e_32.append(np.linalg.norm(Y32[:, j] - y64) / np.linalg.norm(y64))
    print(f"tensor-core vs FP64: max {max(e_tc):.2e}; CUDA-core FP32 vs FP64: max {max(e_32):.2e}")
    # Both FP32 forms carry the FP32 operator's error against FP64: folding
    # Atilde^-1 into the blocks leaves cancellation that FP32 rounding feeds,
    # up to ~5e-5 (the bound of the single-vector FP32 tests). The
    # tensor-core form (three TF32 products, FP32 accumulation) must be no
    # less accurate than the CUDA-core FP32 form.
    assert max(e_tc) <= 5e-5
    assert max(e_tc) <= 2.0 * max(e_32) + 1e-7
    op.close()


def test_batched_solver_tensor_core_blocks_match_cuda_core_blocks(ls, ora):
    cfg = full_cfg(CFG_C1)
    op = ls.Operator(cfg, device=0)
    op.enable_f32()
    thetas = 2 * np.pi * np.arange(64) / 64
    B = op.rhs_angles(thetas)
    op.set_batch_width(64)
    X64, n64, rr64, c64 = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
    op.set_batch_width(8)
    X8, n8, rr8, c8 = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
    assert c64 == ls.LS_OK and c8 == ls.LS_OK
    assert np.max(rr64) <= 1e-8 and np.max(rr8) <= 1e-8
    ref = ora.Oracle(cfg.as_dict())
    for j in (0, 17, 63):
        r = np.linalg.norm(B[:, j] - ref.matvec(X64[:, j])) / np.linalg.norm(B[:, j])
        assert r <= 1.5e-8, (j, r)
        assert np.linalg.norm(X64[:, j] - X8[:, j]) / np.linalg.norm(X8[:, j]) <= 1e-7
    op.close()
