"""Programmatic dependent launch (PDL) of the kernel chains.

1. tests/cuda/pdl_coherence_probe.cu provokes the pattern in which a chained
   kernel can read stale data: it becomes resident while the kernel two
   launches before still reads a buffer on the same SM, and the kernel in
   between rewrites that buffer. The library reads every chain-produced
   value with ld.global.cg (csrc/launch.h, ld_chain); with that load the
   probe must see no stale value. The other load forms are reported.
2. The level-6 benchmark operator gives bitwise identical results with PDL
   and with plain stream-ordered launches: back-to-back matvecs of all three
   kernel families on different inputs, restarted GMRES and the
   mixed-precision solve.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="needs nvcc")
def test_pdl_probe_sees_no_stale_value_with_the_librarys_load(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "pdl_probe")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", exe,
                    os.path.join(ROOT, "tests", "cuda", "pdl_coherence_probe.cu")], check=True, timeout=600)
    out = subprocess.run([exe, "2000"], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = re.findall(r"pdl=(\d) reader=(\S+) check=(\S+) rounds=\d+ stale=(\d+)", out.stdout)
    assert len(rows) == 12
    for pdl, reader, check, stale in rows:
        if check == "ld.global.cg" or pdl == "0":
            assert int(stale) == 0, (pdl, reader, check, stale)


def _workload(ls):
    return ls.Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=10, degreeOfBases=6, nLevelsUniform=6,
                     Qchoice=6, findPhi=1, reference_rounding=1, L=1.0, kappa=40.0,
                     bumps=ls.seeded_bumps(20261203))


def _run_all(ls, op, xs):
    torch = pytest.importorskip("torch")
    out = []
    xd = [torch.from_numpy(x).cuda() for x in xs]
    for kernels in (ls.LS_F64_NATIVE, ls.LS_F64_DOUBLE_FLOAT):
        op.set_f64_kernels(kernels)
        ys = [torch.empty_like(v) for v in xd]
        for v, y in zip(xd, ys):  # back to back, no host synchronisation in between
            op.matvec_device(v.data_ptr(), y.data_ptr(), 0)
        ys32 = [torch.empty_like(v) for v in xd]
        for v, y in zip(xd, ys32):
            op.matvec_device(v.data_ptr(), y.data_ptr(), 0, precision=ls.LS_PREC_F32)
        torch.cuda.synchronize()
        out += [y.cpu().numpy() for y in ys + ys32]
    op.set_f64_kernels(ls.LS_F64_NATIVE)
    b = op.rhs()
    out.append(op.gmres_restarted(b, 10, 1))
    out.append(op.gmres_mixed(b, max_outer=10, inner_iter=100, tol=1e-8)[0])
    return out


def test_pdl_and_plain_launches_are_bitwise_equal_at_level6(ls):
    op = ls.Operator(_workload(ls), device=0)
    op.enable_f32()
    rng = np.random.default_rng(99)
    xs = [rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N) for _ in range(3)]
    was = ls.get_pdl()
    try:
        ls.set_pdl(True)
        with_pdl = _run_all(ls, op, xs)
        ls.set_pdl(False)
        plain = _run_all(ls, op, xs)
    finally:
        ls.set_pdl(was)
    assert len(with_pdl) == len(plain) == 14
    for k, (a, b) in enumerate(zip(with_pdl, plain)):
        assert np.array_equal(a, b), f"result {k} differs between PDL and plain launches"
    op.close()


def test_overlapped_and_serial_near_field_are_bitwise_equal_at_level6(ls):
    """The native FP64 matvec with its near field on a second stream beside
    the far-field chain (the default) and after it (ls_set_near_overlap(0)):
    back-to-back matvecs on different inputs, restarted GMRES and the
    mixed-precision solve give the same bits; with PDL on and off."""
    op = ls.Operator(_workload(ls), device=0)
    op.enable_f32()
    rng = np.random.default_rng(7)
    xs = [rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N) for _ in range(3)]
    was, was_pdl = ls.get_near_overlap(), ls.get_pdl()
    try:
        runs = {}
        for pdl in (True, False):
            ls.set_pdl(pdl)
            for overlap in (True, False):
                ls.set_near_overlap(overlap)
                runs[(pdl, overlap)] = _run_all(ls, op, xs)
    finally:
        ls.set_near_overlap(was)
        ls.set_pdl(was_pdl)
    ref = runs[(True, False)]
    for key, res in runs.items():
        for k, (a, b) in enumerate(zip(res, ref)):
            assert np.array_equal(a, b), f"result {k} differs (pdl, overlap) = {key}"
    op.close()
