"""The two tensor-core block-apply kernels of csrc/batched_tc.cu against each
other: the warp-specialized tc_ws_kernel (the default: loader, converter,
MMA and epilogue warps fed by per-CTA stage programs) and the two-CTA
tc_gemm_kernel (LS_TC_WS=0). Both issue the same MMAs per stage and add the
accumulator chunks into the running sums in the same order, so their
outputs agree bit for bit. The kernel is chosen once per process, so each
runs in a child process of its own; the phases covered are the uniform
tree's (upward, M2L, downward, factored near field with find_phi on and
off) and the adaptive tree's generic near phase."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import CFG_C1, CFG_HFR, CFG_L5_BUMPS, ROOT, full_cfg

pytestmark = pytest.mark.gpu

README = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=5, Qchoice=0,
              findPhi=1, reference_rounding=1, L=0.5, kappa=40.0, tree_adaptive=1, treeAdaptivity=5)

CHILD = r"""
import sys, json, numpy as np
sys.path.insert(0, sys.argv[1])
import lippmann_schwinger_solver_gb300 as ls
cfg = json.loads(sys.argv[2])
op = ls.Operator(ls.Config(**cfg), device=0)
op.enable_f32()
rng = np.random.default_rng(11)
X = np.asfortranarray(rng.uniform(-1, 1, (op.N, 64)) + 1j * rng.uniform(-1, 1, (op.N, 64)))
np.save(sys.argv[3], op.matvec_f32_many(X))
op.close()
"""


def _apply(cfg, ws, path):
    import dataclasses
    import json
    if dataclasses.is_dataclass(cfg):
        cfg = dataclasses.asdict(cfg)
    env = dict(os.environ, LS_TC_WS=str(ws))
    out = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(cfg), path], env=env, capture_output=True,
                         text=True, timeout=900)
    assert out.returncode == 0, out.stdout + out.stderr
    return np.load(path)


@pytest.mark.parametrize("cfg", [full_cfg(CFG_L5_BUMPS), full_cfg(CFG_HFR, findPhi=0), README],
                         ids=["uniform-level5", "uniform-hfr-nophi", "adaptive-readme"])
def test_warp_specialized_kernel_equals_two_cta_kernel(tmp_path, cfg):
    y_ws = _apply(cfg, 1, str(tmp_path / "ws.npy"))
    y_2c = _apply(cfg, 0, str(tmp_path / "two_cta.npy"))
    diff = float(np.max(np.abs(y_ws - y_2c)) / np.max(np.abs(y_2c)))
    print(f"max |warp-specialized - two-CTA| / max |y| = {diff:.2e}")
    assert np.all(np.isfinite(y_ws))
    assert np.array_equal(y_ws, y_2c)


def test_mma_issue_cost_and_stage_count(ls):
    """ls_measure_mma_issue: below N = 128 one TF32 MMA costs the same
    whatever N (the floor of the block apply), at N = 256 the tensor rate
    makes it dearer; ls_op_tc_stages counts the stages of the tensor-core
    form once the first 64-wide apply has built it."""
    c16, c64, c256 = (ls.measure_mma_issue(0, n) for n in (16, 64, 256))
    print(f"cycles per MMA: N=16 {c16:.1f}, N=64 {c64:.1f}, N=256 {c256:.1f}")
    assert 5.0 < c16 < 1000.0 and c64 < 1.5 * c16 and c256 > 1.5 * c16
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    op.enable_f32()
    assert op.tc_stages() == 0
    op.time_block_apply(64, warmup=0, iters=1)
    assert op.tc_stages() > 0
    op.close()


def test_bounded_wait_gives_up_and_the_context_survives(ls):
    """Failure detection without a GPU fault: the tensor-core kernels' bounded
    mbarrier wait, run on a barrier that nothing arrives on (a short poll
    limit), gives up and records it; the probe frees its tensor memory, and
    the same process then runs a tensor-core block apply normally."""
    assert ls.tc_wait_probe(0, polls=100000)
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    op.enable_f32()
    assert op.time_block_apply(64, warmup=1, iters=2) > 0.0
    op.close()
