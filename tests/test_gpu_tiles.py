"""Tile shapes chosen through the autotuner's knobs (LS_TILE_<kind> =
"rows,warps") change how the phases are packed, not the operator: the
matvec stays within rounding of the default packing and within the parity
bar of the oracle."""
import os

import numpy as np
import pytest

from conftest import CFG_HFR, full_cfg

pytestmark = pytest.mark.gpu


def test_tile_knobs_keep_the_operator(ls, ora, monkeypatch):
    cfg = full_cfg(CFG_HFR)
    rng = np.random.default_rng(11)
    op = ls.Operator(cfg, device=0)
    x = rng.uniform(-1, 1, op.N) + 1j * rng.uniform(-1, 1, op.N)
    y0 = op.matvec(x)
    op.close()
    for knobs in ({"M2L": "2,24", "UP": "4,96", "DOWN": "1,48"}, {"M2L": "8,96", "UP": "1,24", "DOWN": "8,24"}):
        for k, v in knobs.items():
            monkeypatch.setenv("LS_TILE_" + k, v)
        op = ls.Operator(cfg, device=0)
        y = op.matvec(x)
        op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
        ydf = op.matvec(x)
        op.close()
        assert np.linalg.norm(y - y0) / np.linalg.norm(y0) < 1e-13
        assert np.linalg.norm(ydf - y0) / np.linalg.norm(y0) < 2e-11
    yo = ora.Oracle(cfg.as_dict()).matvec(x)
    assert np.linalg.norm(y0 - yo) / np.linalg.norm(yo) < 1e-10
