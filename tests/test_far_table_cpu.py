"""The far-field sum table of ls_config.far_on_gpu, tabulated on the host
cores (an operator without a device), against the oracle.

The table indexes a far-field entry by the distinct values of the x and y
parts of (target - leaf centre); each record is the host's own 31-term sum
for exactly those bits, so an assembly that reads every entry from it must
be the default one bit for bit: the same NCA skeletons at every level and
cone (ACA_only_nodes, GMRES/ACA.hpp:253-481), the same moments and near
blocks. Mode 2 (NCA on the GPU) without a device runs the host's NCA on the
table. A wrong index in the tables would change entries and with them the
skeletons."""
import os

import numpy as np
import pytest

from conftest import CFG_C1, CFG_HFR, CFG_L5_BUMPS, full_cfg


@pytest.mark.parametrize("base", [CFG_C1, CFG_HFR, CFG_L5_BUMPS], ids=["c1", "hfr-cones", "level5-kappa40"])
@pytest.mark.parametrize("mode", [1, 2])
def test_host_tabulated_far_field_equals_oracle(ls, ora, base, mode):
    if base is CFG_L5_BUMPS and mode == 2:
        pytest.skip("the level-5 tree is covered in mode 1; mode 2 runs the same host code without a device")
    cfg = full_cfg(base, far_on_gpu=mode)
    op = ls.Operator(cfg, device=-1)
    ref = ora.Oracle(cfg.as_dict())
    assert np.array_equal(op.skeleton_dump(), ref.skeleton_dump())
    M, B = op.precomputations()
    assert np.array_equal(M, ref.far_moments())
    assert np.array_equal(B, ref.near_blocks())
    assert ls.skeleton_agreement(op.skeleton_dump(), ref.skeleton_dump()) == 1.0
    ref.close()
    op.close()


def test_skeleton_parser_round_trip(ls):
    op = ls.Operator(full_cfg(CFG_C1), device=-1)
    dump = op.skeleton_dump()
    nodes = ls.skeleton_nodes(dump)
    info = op.info
    n_nodes = sum((1 << (2 * j)) * (1 if j >= info["level_LFR"] else 16 * 2 ** (info["level_LFR"] - 1 - j))
                  for j in range(2, info["n_levels"] + 1))
    assert len(nodes) == n_nodes
    rebuilt = []
    for (j, k, cn), v in nodes.items():
        rebuilt += [j, k, cn, v[0], v[1]]
        for lst in v[2:]:
            rebuilt += [len(lst)] + list(lst)
    assert np.array_equal(np.array(rebuilt, dtype=np.int32), dump)
    # One changed skeleton index: exactly one node disagrees.
    key = next(k for k, v in nodes.items() if len(v[2]) > 0)
    changed = dict(nodes)
    v = list(changed[key])
    v[2] = (v[2][0] + 1,) + v[2][1:]
    changed[key] = tuple(v)
    moved = []
    for (j, k, cn), v in changed.items():
        moved += [j, k, cn, v[0], v[1]]
        for lst in v[2:]:
            moved += [len(lst)] + list(lst)
    assert ls.skeleton_agreement(np.array(moved, dtype=np.int32), dump) == pytest.approx(1.0 - 1.0 / len(nodes))
    op.close()


@pytest.mark.parametrize("base", [CFG_C1, CFG_HFR, CFG_L5_BUMPS], ids=["c1", "hfr-cones", "level5-kappa40"])
def test_table_filled_m2l_tiles_equal_the_default_packing(ls, tmp_path, base):
    """far_on_gpu = 3 forms the M2L tiles from tile descriptors and the
    far-field table (on the device, or on the host without one) instead of
    packing host-filled blocks. Run on the host by
    tests/cpp/packed_program_check.cpp (every access checked in bounds), the
    far part of the matvec (upward, M2L, downward phases) equals the
    default packing's bit for bit."""
    import subprocess
    from conftest import ROOT
    exe = str(tmp_path / "packed_program_check")
    src = os.path.join(ROOT, "tests", "cpp", "packed_program_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                    src, "-o", exe], check=True, capture_output=True, timeout=600)
    rng = np.random.default_rng(3)
    ys = {}
    for mode in (0, 3):
        cfg = full_cfg(base, far_on_gpu=mode)
        cfg_path, x_path, y_path = (str(tmp_path / f"{n}{mode}.bin") for n in ("cfg", "x", "y"))
        with open(cfg_path, "wb") as f:
            f.write(bytes(cfg.to_c()))
        n = (1 << (2 * cfg.nLevelsUniform)) * cfg.nChebNodes ** 2
        if mode == 0:
            x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
        x.astype(np.complex128).tofile(x_path)
        out = subprocess.run([exe, cfg_path, x_path, y_path, "--far-only"], capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stdout + out.stderr
        ys[mode] = np.fromfile(y_path, dtype=np.complex128)
    assert np.linalg.norm(ys[0]) > 0 and np.array_equal(ys[3], ys[0])


@pytest.mark.parametrize("over", [dict(findPhi=0), dict(nChebNodes=4, degreeOfBases=4), dict(reference_rounding=0)],
                         ids=["bare-helmholtz", "4x4-nodes", "unrounded"])
def test_host_tabulated_far_field_other_operators(ls, ora, over):
    """The table's indexing for other node counts (rank 16: x rows of 4
    nodes), the bare Helmholtz operator (no kappa^2 q scaling) and unrounded
    moments: the assembly stays the oracle's bit for bit, table fill of the
    M2L tiles included (mode 3 without a device)."""
    cfg = full_cfg(CFG_HFR, far_on_gpu=3, **over)
    op = ls.Operator(cfg, device=-1)
    ref = ora.Oracle(cfg.as_dict())
    assert np.array_equal(op.skeleton_dump(), ref.skeleton_dump())
    M, B = op.precomputations()
    assert np.array_equal(M, ref.far_moments()) and np.array_equal(B, ref.near_blocks())
    ref.close()
    op.close()
