"""Regenerates the golden fixtures in this folder from the CPU oracle.

The reference itself cannot be built here (Eigen and Boost.Math are
missing), so these vectors are outputs of the oracle's restatement of the
reference DAFMM. They freeze its results: tests check that the oracle keeps
reproducing them and that the GPU path matches them.

One set per host architecture (tests/golden/<machine>/): glibc's libm
differs in the last bit between x86-64 and aarch64, which can move an NCA
pivot at a near-tie and hence change the operator at the NCA tolerance.

    python tests/golden/make_golden.py
"""
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402

CASES = {
    # uniform level 3, kappa 10, Gaussian contrast 1.5 exp(-160|x|^2), NCA 1e-8
    "l3_k10_gauss": dict(nLevelsUniform=3, kappa=10.0, TOL_POW=8, Qchoice=0),
    # the 256-leaf CPU-runnable configuration (level 4, kappa 10, NCA 1e-8)
    "l4_k10_gauss": dict(nLevelsUniform=4, kappa=10.0, TOL_POW=8, Qchoice=0),
    # directional (HFR cones at level 2), flat-bump contrast, NCA 1e-10
    "l4_k24_flatbump": dict(nLevelsUniform=4, kappa=24.0, TOL_POW=10, Qchoice=3),
}
BASE = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, degreeOfBases=6, findPhi=1, reference_rounding=1, L=1.0)


def main():
    out = os.path.join(HERE, platform.machine())
    os.makedirs(out, exist_ok=True)
    for name, over in CASES.items():
        cfg = dict(BASE, **over)
        o = oracle.Oracle(cfg)
        rng = np.random.default_rng(12345)
        x = rng.uniform(-1, 1, o.N) + 1j * rng.uniform(-1, 1, o.N)
        y = o.matvec(x)
        b = o.rhs()
        xs, hist, it = o.gmres(b, 200, 1e-10)
        ranks = np.array([o.level_lfr, o.nlevels, len(o.skeleton_dump())])
        np.savez_compressed(os.path.join(out, name + ".npz"), x=x, y=y, b=b, x_gmres=xs, gmres_iters=it,
                            ranks=ranks, skeleton=o.skeleton_dump(), cfg=np.array(repr(cfg)))
        print(name, o.N, it)


if __name__ == "__main__":
    main()
