"""The precomputation cache (ls_set_precompute_cache, csrc/assemble.cpp):
records of the far moments M and the near blocks, in memory or as binary
files, in place of the reference's 6-digit text files that it recomputes on
every run (G_FMM2DTree.hpp:1264-1270, 1868-1950).

A record holds the exact values an assembly computed, keyed on everything
they depend on, so an assembly that reads it must be the oracle's bit for
bit; a record is reused across processes through its file; a file that does
not match its key is ignored (the assembly integrates again and stays
exact); a different wavenumber or leaf size misses."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import CFG_C1, CFG_L5_BUMPS, ROOT, full_cfg

SMALL_ADAPTIVE = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=5,
                      Qchoice=0, findPhi=1, reference_rounding=1, L=0.5, kappa=10.0, tree_adaptive=1,
                      treeAdaptivity=3)


@pytest.fixture
def cache(ls):
    yield ls
    ls.set_precompute_cache(None)


def _same_as_oracle(ls, ora, cfg, op):
    ref = ora.Oracle(cfg.as_dict())
    ok = np.array_equal(op.skeleton_dump(), ref.skeleton_dump())
    M, B = op.precomputations()
    ok = ok and np.array_equal(M, ref.far_moments()) and np.array_equal(B, ref.near_blocks())
    ref.close()
    return ok


@pytest.mark.parametrize("base", [CFG_C1, CFG_L5_BUMPS], ids=["c1", "level5-kappa40"])
def test_memory_cache_hits_and_stays_exact(cache, ora, base):
    ls = cache
    cfg = full_cfg(base)
    ls.set_precompute_cache("")
    h0, m0 = ls.precompute_cache_stats()
    a = ls.Operator(cfg, device=-1)
    h1, m1 = ls.precompute_cache_stats()
    b = ls.Operator(cfg, device=-1)
    h2, m2 = ls.precompute_cache_stats()
    assert (h1 - h0, m1 - m0) == (0, 1) and (h2 - h1, m2 - m1) == (1, 0)
    assert b.info["assemble_stage_seconds"][1] < a.info["assemble_stage_seconds"][1]
    assert _same_as_oracle(ls, ora, cfg, b)
    # Another wavenumber is another record.
    c = ls.Operator(full_cfg(base, kappa=cfg.kappa + 1.0), device=-1)
    assert ls.precompute_cache_stats()[1] == m2 + 1
    for op in (a, b, c):
        op.close()


CHILD = r"""
import sys, json
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import numpy as np
import lippmann_schwinger_solver_gb300 as ls
from conftest import CFG_C1, full_cfg
ls.set_precompute_cache(sys.argv[2])
op = ls.Operator(full_cfg(CFG_C1), device=-1)
M, B = op.precomputations()
np.save(sys.argv[3], np.concatenate([M.ravel(), B.ravel()]))
np.save(sys.argv[4], op.skeleton_dump())
print(json.dumps(ls.precompute_cache_stats()))
"""


def _child(tmp_path, d, tag):
    out = subprocess.run([sys.executable, "-c", CHILD, ROOT, str(d), str(tmp_path / f"mb{tag}.npy"),
                          str(tmp_path / f"sk{tag}.npy")], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    import json
    return tuple(json.loads(out.stdout.strip().splitlines()[-1])), np.load(tmp_path / f"mb{tag}.npy"), \
        np.load(tmp_path / f"sk{tag}.npy")


def test_file_cache_across_processes_and_bad_files(ls, ora, tmp_path):
    d = tmp_path / "lspc"
    d.mkdir()
    st1, mb1, sk1 = _child(tmp_path, d, 1)
    assert tuple(st1) == (0, 1)
    files = sorted(os.listdir(d))
    assert len(files) == 1 and files[0].endswith(".lspc")
    st2, mb2, sk2 = _child(tmp_path, d, 2)  # a fresh process reads the file
    assert tuple(st2) == (1, 0)
    assert np.array_equal(mb1, mb2) and np.array_equal(sk1, sk2)
    ref = ora.Oracle(full_cfg(CFG_C1).as_dict())
    assert np.array_equal(sk2, ref.skeleton_dump())
    ref.close()
    # A damaged file (one value changed, or cut short) is ignored.
    p = d / files[0]
    raw = bytearray(p.read_bytes())
    raw[-3] ^= 0xFF
    p.write_bytes(bytes(raw[:-16]))
    st3, mb3, sk3 = _child(tmp_path, d, 3)
    assert tuple(st3) == (0, 1)
    assert np.array_equal(mb3, mb1) and np.array_equal(sk3, sk1)
    st4, _, _ = _child(tmp_path, d, 4)  # the rewritten file is good again
    assert tuple(st4) == (1, 0)


def test_adaptive_tree_records(cache, ora):
    ls = cache
    ls.set_precompute_cache("")
    h0, m0 = ls.precompute_cache_stats()
    a = ls.Operator(ls.Config(**SMALL_ADAPTIVE), device=-1)
    h1, m1 = ls.precompute_cache_stats()
    b = ls.Operator(ls.Config(**SMALL_ADAPTIVE), device=-1)
    h2, m2 = ls.precompute_cache_stats()
    assert h1 == h0 and m1 > m0          # every leaf level's M and every near block integrated once
    assert h2 - h1 == m1 - m0 and m2 == m1
    assert np.array_equal(a.skeleton_dump(), b.skeleton_dump())
    assert b.info["assemble_stage_seconds"][1] < 0.1 * a.info["assemble_stage_seconds"][1]
    from test_adaptive_cpu import _oracle_skeletons
    assert np.array_equal(b.skeleton_dump(), _oracle_skeletons(ora, SMALL_ADAPTIVE, 3))
    a.close()
    b.close()


def test_cache_off_by_default_and_stats_checked(ls):
    ls.set_precompute_cache(None)
    h0, m0 = ls.precompute_cache_stats()
    op = ls.Operator(full_cfg(CFG_C1), device=-1)
    op.close()
    assert ls.precompute_cache_stats() == (h0, m0)
    assert ls.lib().ls_precompute_cache_stats(None, None) == ls.LS_E_INVALID


def test_unwritable_directory_keeps_memory_records(cache, ora, tmp_path):
    """A cache directory that cannot be written (here: a path below a plain
    file) costs nothing but the files: assemblies still succeed, stay the
    oracle's bit for bit, and the records held in memory still hit."""
    ls = cache
    blocker = tmp_path / "not_a_dir"
    blocker.write_text("x")
    ls.set_precompute_cache(str(blocker / "sub"))
    cfg = full_cfg(CFG_C1)
    h0, m0 = ls.precompute_cache_stats()
    a = ls.Operator(cfg, device=-1)
    b = ls.Operator(cfg, device=-1)
    h1, m1 = ls.precompute_cache_stats()
    assert (h1 - h0, m1 - m0) == (1, 1)
    assert _same_as_oracle(ls, ora, cfg, b)
    a.close()
    b.close()
