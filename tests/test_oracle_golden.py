"""The CPU oracle against the reference's golden trajectories.

Mirrors the reference tests that hold these files:
  test_osecir.py:122-150, test_osecir_ageres.py:116-145 (default Cash-Karp 5(4))
  test_odesecir_ageres.cpp:110-189 (Cash-Karp, dt in [0.3, 1])
  test_odesecir.cpp:39-112, test_odesecir_ageres.cpp:27-108 (RKF45)
Same tolerances as the reference (absolute, on group sums).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.scenarios import GOLDEN_CASES, golden_case, sum_groups


@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_oracle_matches_golden(name):
    c = golden_case(name)
    t, y, st = O.simulate(c["model"], 0, c["t0"], c["tmax"], c["dt"], c["opts"])
    exp = c["expected"]
    assert len(t) == exp.shape[0]
    np.testing.assert_allclose(t, exp[:, 0], rtol=0, atol=c["tol"])
    np.testing.assert_allclose(sum_groups(y, c["G"]), exp[:, 1:], rtol=0, atol=c["tol"])


def test_golden_time_grid_is_adaptive():
    # default Cash-Karp grows 0.1 -> 0.45 (factor 0.9*5 cap) on the first accepted step
    c = golden_case("py_osecir_ck54")
    t, _, st = O.simulate(c["model"], 0, c["t0"], c["tmax"], c["dt"], c["opts"])
    assert t[1] == pytest.approx(0.1) and t[2] == pytest.approx(0.55)
    assert st["rejected_steps"] > 0  # the golden grid includes rejected attempts


def test_population_conserved():
    # test_odesecir.cpp:126-181: the total stays 10000 within 1e-10
    c = golden_case("py_osecir_ageres_ck54")
    _, y, _ = O.simulate(c["model"], 0, 0.0, 50.0, 0.1, c["opts"])
    np.testing.assert_allclose(y.sum(axis=1), 10000.0, rtol=0, atol=1e-9)


def test_zero_population_no_nan():
    # test_odesecir.cpp:586-602
    c = golden_case("py_osecir_ck54")
    m = c["model"].with_init_state(np.zeros(10))
    dydt = O.eval_rhs(m, 0, np.zeros(10), np.zeros(10), 0.0)
    assert np.all(np.isfinite(dydt)) and np.all(dydt == 0)
