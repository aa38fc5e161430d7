"""Many right-hand sides on one operator (ls_gmres_mixed_batched).

Each column stops on its own FP64 true residual, like ls_gmres_mixed;
the batched solution must agree with the single-vector FP64 GMRES solution
to the accuracy both solves carry (residual 1e-8, relative solution
difference bound 1e-5 written below).
"""
import numpy as np
import pytest

from conftest import CFG_C1, CFG_HFR, CFG_L3_K10, full_cfg

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("base,over,kernels", [(CFG_C1, {}, 0), (CFG_HFR, {}, 1), (CFG_L3_K10, {"nChebNodes": 8}, 1)])
def test_batched_solve_matches_single_solves(ls, base, over, kernels):
    op = ls.Operator(full_cfg(base, **over), device=0)
    op.enable_f32()
    op.set_f64_kernels(kernels)
    thetas = np.linspace(0.0, 2 * np.pi, 11, endpoint=False)  # one full block of 8 and a partial one
    B = op.rhs_angles(thetas)
    assert np.allclose(B[:, 0], op.rhs(), rtol=1e-14, atol=0)
    X, nmv, rr, code = op.gmres_mixed_batched(B, max_outer=20, inner_iter=200, tol=1e-8)
    assert code == 0
    assert nmv > 0
    assert np.all(rr <= 1e-8)
    op.set_f64_kernels(ls.LS_F64_NATIVE)
    for j in (0, 3, 8, 10):
        r = B[:, j] - op.matvec(X[:, j])
        assert np.linalg.norm(r) / np.linalg.norm(B[:, j]) <= 1.5e-8
        xs, _, _, rs, cs = op.gmres(B[:, j], max_iter=400, tol=1e-10)
        assert cs == 0
        assert _rel(X[:, j], xs) <= 1e-5
    op.close()


def test_batched_rejects_bad_input(ls):
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    B = op.rhs_angles([0.0, 1.0])
    with pytest.raises(ls.LSError):  # FP32 operator not enabled
        op.gmres_mixed_batched(B)
    op.enable_f32()
    with pytest.raises(ValueError):
        op.gmres_mixed_batched(B[:-1])
    op.close()


@pytest.mark.parametrize("workers", [1, 2])
def test_many_scatterers_pipeline(ls, workers):
    """Several scatterers of different size and wavenumber, each with many
    directions; assembly of the next overlaps the solve of the current one
    (workers = 1), or a work queue assembles and solves two at a time
    (workers = 2, solves of different operators in flight together). Every
    direction of every scatterer meets the FP64 tolerance, and the solutions
    equal those of the same solve run alone."""
    from lippmann_schwinger_solver_gb300 import scatterers as sc
    specs = [(3, 12.0, ((0.1, -0.2, 1.0, 0.15),)), (4, 30.0, ((-0.3, 0.2, 0.8, 0.1), (0.4, 0.1, 1.2, 0.07))),
             (3, 20.0, ((0.2, 0.3, 1.1, 0.12),))]
    recs, total, sols = sc.solve_many(specs, angles=16, tol=1e-8, keep_solutions=True, workers=workers)
    assert total["all_converged"] and total["max_true_residual"] <= 1e-8
    assert [r["N"] for r in recs] == [2304, 9216, 2304]
    assert [r["scatterer"] for r in recs] == [0, 1, 2]
    op = ls.Operator(sc.config(*specs[1]), device=0)
    op.enable_f32()
    B = op.rhs_angles(2 * np.pi * np.arange(16) / 16)
    X, _, rr, code = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
    assert code == ls.LS_OK
    assert np.linalg.norm(X - sols[1]) / np.linalg.norm(X) < 1e-12
    op.close()


def test_operators_of_different_sizes_share_the_kernels(ls):
    """The tensor-core kernels' dynamic shared-memory limit is one setting
    per kernel for the process: setting up a smaller operator's tensor-core
    form after a larger one's must not lower it under the larger one's
    launches (it did, and the larger operator's next batched solve failed
    with an invalid-argument launch error when two scatterers of different
    sizes were solved from two threads)."""
    from conftest import CFG_L5_BUMPS
    big = ls.Operator(full_cfg(CFG_L5_BUMPS), device=0)
    big.enable_f32()
    big.time_block_apply(64, warmup=0, iters=1)
    small = ls.Operator(full_cfg(CFG_L3_K10), device=0)
    small.enable_f32()
    small.time_block_apply(64, warmup=0, iters=1)
    for op in (big, small):
        B = op.rhs_angles(2 * np.pi * np.arange(8) / 8)
        X, nmv, rr, code = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
        assert code == ls.LS_OK and np.max(rr) <= 1e-8
    big.close()
    small.close()
