"""The many-scatterer pipeline's host logic (lippmann_schwinger_solver_gb300
/scatterers.py) without a GPU: operators assembled without a device refuse
the FP32 copy (LS_E_STATE), so every scatterer fails. Both schedules must
raise that error, and the work queue (workers > 1) must stop its builders
and free what they built instead of waiting for solves that never come."""
import pytest

SPECS = [(3, 12.0, ((0.1, -0.2, 1.0, 0.15),)), (3, 20.0, ((0.2, 0.3, 1.1, 0.12),))] * 3


@pytest.mark.timeout(300)
@pytest.mark.parametrize("workers", [1, 2, 3])
def test_pipeline_raises_the_first_failure(ls, workers):
    from lippmann_schwinger_solver_gb300 import scatterers as sc
    with pytest.raises(ls.LSError) as ei:
        sc.solve_many(SPECS, angles=4, device=-1, workers=workers)
    assert ei.value.code == ls.LS_E_STATE


def test_scatterer_specs_are_seeded_and_in_range():
    from lippmann_schwinger_solver_gb300 import scatterers as sc
    a, b = sc.scatterer_specs(32, 7), sc.scatterer_specs(32, 7)
    assert a == b and len(a) == 32
    for level, kappa, bumps in a:
        assert level in (4, 5, 6) and 10.0 <= kappa <= 60.0 and 1 <= len(bumps) <= 4
