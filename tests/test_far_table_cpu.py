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
