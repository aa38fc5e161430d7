"""Far-field assembly on the GPU (ls_config.far_on_gpu, csrc/far_gpu.cu)
against the host assembler, which is the oracle's bit for bit.

Mode 1 tabulates the far-field sums of every distinct relative position on
the GPU and leaves the NCA (ACA_only_nodes, GMRES/ACA.hpp:253-481) on the
host; mode 2 also runs the NCA on the GPU, one thread block per NCA block.
The GPU's Bessel, trigonometric and hypot values differ from the host's in
the last bits. On a uniform tree many pivot candidates are equal in magnitude up to
such bits (mirror-image positions), so those ties break differently: the
skeletons are other valid choices, not the oracle's. The bar is therefore
the assembly's own sensitivity: the GPU-assembled operator's matvec is no
farther from the host's than 3x the distance between the host operators at
NCA tolerances TOL and TOL/10 (the reference's compressed operator moves
that much from a legitimate change of skeletons; at level 5, kappa 40 it
moves by about 3%, on the level-4 kappa-24 tree by 1.4e-8). Also printed:
the skeleton agreement rates; asserted: GMRES converging on the
GPU-assembled operator and, on the level-5 tree, the GPU NCA stage faster
than the host's. The same table tabulated on the host is bit-exact with the
oracle (tests/test_far_table_cpu.py)."""
import numpy as np
import pytest

from conftest import CFG_C1, CFG_HFR, CFG_L5_BUMPS, full_cfg

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("base", [CFG_C1, CFG_HFR, CFG_L5_BUMPS], ids=["c1", "hfr-cones", "level5-kappa40"])
def test_far_assembly_on_gpu_against_host(ls, ora, base):
    cfg = full_cfg(base)
    tol = 10.0 ** -cfg.TOL_POW
    host = ls.Operator(cfg, device=0)
    tighter = ls.Operator(full_cfg(base, TOL_POW=cfg.TOL_POW + 1), device=0)
    o = ora.Oracle(cfg.as_dict())
    rng = np.random.default_rng(23)
    x = rng.uniform(-1, 1, host.N) + 1j * rng.uniform(-1, 1, host.N)
    y_host = host.matvec(x)
    d_tol = _rel(y_host, tighter.matvec(x))
    skel_host = host.skeleton_dump()
    assert np.array_equal(skel_host, o.skeleton_dump())
    assert _rel(y_host, o.matvec(x)) <= 1e-12
    res = {}
    for mode in (1, 2):
        op = ls.Operator(full_cfg(base, far_on_gpu=mode), device=0)
        y = op.matvec(x)
        res[mode] = dict(vs_host=_rel(y, y_host),
                         agree=ls.skeleton_agreement(op.skeleton_dump(), skel_host), skel=op.skeleton_dump(),
                         nca_s=op.info["assemble_stage_seconds"][3], pack_s=op.info["assemble_stage_seconds"][5])
        b = op.rhs()
        xs, hist, it, rr, code = op.gmres(b, 300, 1e-10)
        res[mode]["gmres"] = (code, it, rr)
        op.close()
    a21 = ls.skeleton_agreement(res[2]["skel"], res[1]["skel"])
    nca_host, pack_host = host.info["assemble_stage_seconds"][3], host.info["assemble_stage_seconds"][5]
    print(f"tol {tol:.0e}: host NCA {nca_host:.3f} s, pack {pack_host:.3f} s; host operators at tol and tol/10 "
          f"differ by {d_tol:.2e}")
    for m in (1, 2):
        r = res[m]
        print(f"far_on_gpu={m}: matvec vs host operator {r['vs_host']:.2e} ({r['vs_host'] / d_tol:.3f}x the "
              f"tolerance spread), skeleton nodes equal to the host's {r['agree']:.4f}, "
              f"NCA stage {r['nca_s']:.3f} s, pack {r['pack_s']:.3f} s, GMRES {r['gmres']}")
    print(f"mode 2 vs mode 1 skeleton agreement {a21:.4f}")
    for m in (1, 2):
        assert res[m]["vs_host"] <= 3.0 * d_tol
        code, it, rr = res[m]["gmres"]
        assert code == ls.LS_OK and rr <= 2e-10
    if cfg.nLevelsUniform >= 5:
        assert res[2]["nca_s"] < nca_host
    o.close()
    tighter.close()
    host.close()


@pytest.mark.parametrize("base", [CFG_C1, CFG_L5_BUMPS], ids=["c1", "level5-kappa40"])
def test_m2l_tiles_filled_on_the_device(ls, base):
    """far_on_gpu = 3 fills the M2L tiles from the far-field table on the
    device and the operator adopts them; far_on_gpu = 2 packs the same
    entries on the host from the same table. Same skeletons, the same FP64
    matvec bit for bit, and the forms derived from the device tiles (FP32,
    double-float, the 64-wide tensor-core apply) agree as well."""
    rng = np.random.default_rng(31)
    ops = {m: ls.Operator(full_cfg(base, far_on_gpu=m), device=0) for m in (2, 3)}
    x = rng.uniform(-1, 1, ops[2].N) + 1j * rng.uniform(-1, 1, ops[2].N)
    assert np.array_equal(ops[2].skeleton_dump(), ops[3].skeleton_dump())
    y = {m: op.matvec(x) for m, op in ops.items()}
    assert np.array_equal(y[2], y[3])
    for op in ops.values():
        op.enable_f32()
        op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    assert np.array_equal(ops[2].matvec(x), ops[3].matvec(x))
    X = np.asfortranarray(rng.uniform(-1, 1, (ops[2].N, 64)) + 1j * rng.uniform(-1, 1, (ops[2].N, 64)))
    assert np.array_equal(ops[2].matvec_f32_many(X), ops[3].matvec_f32_many(X))
    b = ops[3].rhs()
    xs, hist, it, rr, code = ops[3].gmres(b, 300, 1e-10)
    assert code == ls.LS_OK and rr <= 2e-10
    for op in ops.values():
        op.close()
