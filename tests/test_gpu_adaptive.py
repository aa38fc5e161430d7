"""Adaptive quadtrees on the GPU: the reference's default operator.

At the configuration of the reference's published run (GMRES/Readme.md:43)
the GPU matvec (native FP64 and double-float kernels) equals the oracle's
adaptive restatement to 1e-10, and restarted GMRES on the GPU reproduces
the residuals the README prints (GMRES/Readme.md:64-65, 84-85) to the
printed digits: the GPU product pinned directly to the reference's own
output."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

README = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=5, Qchoice=0,
              findPhi=1, reference_rounding=1, L=0.5, kappa=40.0, tree_adaptive=1, treeAdaptivity=5)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def pair(ls, ora):
    op = ls.Operator(ls.Config(**README), device=0)
    a = ora.AdaptiveOracle(README, treeAdaptivity=5)
    yield op, a
    op.close()
    a.close()


def test_adaptive_matvec_matches_oracle(ls, pair):
    op, a = pair
    assert op.N == a.N == 5328
    for seed in (1, 2):
        rng = np.random.default_rng(seed)
        x = rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N)
        ya = a.matvec(x)
        assert _rel(op.matvec(x), ya) <= 1e-10
        op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
        assert _rel(op.matvec(x), ya) <= 1e-10
        op.set_f64_kernels(ls.LS_F64_NATIVE)


@pytest.mark.parametrize("over", [dict(kappa=20.0, findPhi=0), dict(kappa=20.0, TOL_POW=10, treeAdaptivity=4)])
def test_adaptive_matvec_matches_oracle_on_other_trees(ls, ora, over):
    cfg = dict(README, **over)
    op = ls.Operator(ls.Config(**cfg), device=0)
    a = ora.AdaptiveOracle(cfg, treeAdaptivity=cfg["treeAdaptivity"])
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N)
    ya = a.matvec(x)
    assert _rel(op.matvec(x), ya) <= 1e-10
    op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    assert _rel(op.matvec(x), ya) <= 1e-10
    op.enable_f32()
    torch = pytest.importorskip("torch")
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    op.matvec_device(xt.data_ptr(), yt.data_ptr(), 0, precision=ls.LS_PREC_F32)
    torch.cuda.synchronize()
    assert _rel(yt.cpu().numpy(), ya) <= 5e-5  # the FP32 operator's bound
    op.close()
    a.close()


def test_gpu_restarted_gmres_reproduces_readme_residuals(ls, pair):
    op, a = pair
    b = a.rhs()
    assert np.array_equal(b, op.rhs())
    for restarts, m, published in [(1, 10, 4.59412e-06), (2, 10, 1.28443e-10)]:
        x = op.gmres_restarted(b, m, restarts)
        res = np.linalg.norm(b - op.matvec(x)) / np.linalg.norm(b)
        res_oracle = np.linalg.norm(b - a.matvec(x)) / np.linalg.norm(b)
        assert abs(res / published - 1.0) <= 2e-5, (restarts, m, res)
        assert abs(res_oracle / published - 1.0) <= 2e-5, (restarts, m, res_oracle)


def test_adaptive_solvers_reach_the_fp64_residual(ls, pair):
    op, a = pair
    b = op.rhs()
    x, hist, it, rr, code = op.gmres(b, 200, 1e-10)
    assert code == ls.LS_OK
    assert np.linalg.norm(b - a.matvec(x)) / np.linalg.norm(b) <= 2e-10
    op.enable_f32()
    xm, hm, nmv, rrm, codem = op.gmres_mixed(b, max_outer=10, inner_iter=100, tol=1e-8)
    assert codem == ls.LS_OK
    assert np.linalg.norm(b - a.matvec(xm)) / np.linalg.norm(b) <= 1.5e-8
    assert _rel(xm, x) <= 1e-7


@pytest.mark.parametrize("width", [64, 8])
def test_adaptive_batched_solves(ls, pair, width):
    """Many incidence directions on the adaptive README tree, 64 at a time on
    the tensor cores or 8 on the CUDA cores: the block apply equals the
    single-vector FP32 operator to FP32 accuracy, and every direction reaches
    the FP64 true residual."""
    torch = pytest.importorskip("torch")
    op, _ = pair
    op.enable_f32()
    op.set_batch_width(width)
    rng = np.random.default_rng(19)
    X = np.asfortranarray(rng.uniform(-1, 1, (op.N, width)) + 1j * rng.uniform(-1, 1, (op.N, width)))
    Y = op.matvec_f32_many(X)
    for j in (0, width - 1):
        xt = torch.from_numpy(np.ascontiguousarray(X[:, j])).cuda()
        yt = torch.empty_like(xt)
        op.matvec_device(xt.data_ptr(), yt.data_ptr(), 0, precision=ls.LS_PREC_F32)
        torch.cuda.synchronize()
        assert _rel(Y[:, j], yt.cpu().numpy()) <= 5e-5
    thetas = 2 * np.pi * np.arange(16) / 16
    B = op.rhs_angles(thetas)
    Xs, nmv, rr, code = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
    assert code == ls.LS_OK and np.max(rr) <= 1e-8
    for j in (0, 7):
        assert np.linalg.norm(B[:, j] - op.matvec(Xs[:, j])) / np.linalg.norm(B[:, j]) <= 1.5e-8
    op.set_batch_width(64)
