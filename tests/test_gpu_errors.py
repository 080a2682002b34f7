"""Error behaviour at the C ABI on a GPU: bad arguments and non-finite input
come back as status codes with a message, and the context stays usable."""
import numpy as np
import pytest

from bioshell_gb300 import CrmsdError, synth
from bioshell_gb300.crmsd import CrmsdOptions, Engine

pytestmark = pytest.mark.gpu


def test_nonfinite_input_rejected(engine, golden_small):
    x = golden_small["xyz"].copy()
    x[3, 7, 1] = np.nan
    for prec in ("mixed", "plain64"):
        with pytest.raises(CrmsdError) as ei:
            engine.all_vs_all(x, CrmsdOptions(precision=prec))
        assert ei.value.status == 6
    # the context still works afterwards
    r = engine.all_vs_all(golden_small["xyz"]).values
    assert np.abs(r - golden_small["rmsd"]).max() <= 1e-4


def test_invalid_arguments(engine, enginelib):
    assert enginelib.bs_all_vs_all(engine._h, None, 10, 5, None, None) == 1
    assert enginelib.bs_all_vs_all(engine._h, None, -1, 5, None, None) == 1
    with pytest.raises(CrmsdError):
        engine.pairs(np.zeros((4, 5, 3)), np.array([0, 9]), np.array([1, 2]))
    with pytest.raises(ValueError):
        engine.crmsd(np.zeros((5, 3)), np.zeros((6, 3)))


def test_tiny_sets(engine):
    assert engine.all_vs_all(np.zeros((0, 5, 3))).values.shape == (0,)
    assert engine.all_vs_all(np.zeros((1, 5, 3))).values.shape == (0,)
    sq = engine.all_vs_all(np.ones((1, 5, 3)), CrmsdOptions(layout="square")).values
    assert sq.shape == (1,) and sq[0] == 0.0
    # degenerate structures: all atoms on one point
    r = engine.all_vs_all(np.ones((3, 8, 3)) * np.arange(3)[:, None, None]).values
    np.testing.assert_allclose(r, 0.0, atol=1e-9)


def test_budget_exceeded():
    eng = Engine(0, hbm_budget=1 << 20)
    x = synth.Workload("b", n=400, L=100, seed=1).generate()
    with pytest.raises(CrmsdError) as ei:
        eng.all_vs_all(x)
    assert ei.value.status == 7
    eng.close()
