"""Single-node ODE-SECIR setups of the reference's golden tests, in the
miogpu flat layout, plus loaders for the golden CSV files in this folder.

Setups restated from:
  pycode/memilio-simulation/tests/test_osecir.py:35-85         (1 group, default Cash-Karp)
  pycode/memilio-simulation/tests/test_osecir_ageres.py:35-97  (3 groups, default Cash-Karp)
  cpp/tests/test_odesecir_ageres.cpp:110-189                   (3 groups, Cash-Karp dt in [0.3, 1])
  cpp/tests/test_odesecir.cpp:39-112                           (1 group, RKF45 dt in [0.3, 1])
  cpp/tests/test_odesecir_ageres.cpp:27-108                    (3 groups, RKF45 dt in [0.3, 1])
"""
import os

import numpy as np

from memilio_gb300 import layout as L

HERE = os.path.dirname(os.path.abspath(__file__))


def load_csv(name):
    """Rows of (t, S, E, INS, INSC, ISy, ISyC, ISev, ICri, R, D) summed over age groups."""
    return np.loadtxt(os.path.join(HERE, name), comments="#")


def reference_test_model(G: int, critical_per_severe: float) -> L.GraphArrays:
    """The SECIHURD test model: 10000 people split evenly over G groups,
    contacts 10/G between all groups, damping 0.7 from day 30."""
    fact = 1.0 / G
    p = np.zeros(L.param_stride(G))
    p[L.P_START_DAY] = 60
    p[L.P_SEASONALITY] = 0.2
    p[L.P_ICU_CAPACITY] = L.DBL_MAX
    p[L.P_TNT_CAPACITY] = 35
    p[L.P_TNT_MAX_RISK] = 5.0
    gp = lambda k, v: p.__setitem__(slice(L.group_param_index(k, 0, G), L.group_param_index(k, 0, G) + G), v)
    gp(L.G_TIME_EXPOSED, 3.2)
    gp(L.G_TIME_INS, 2.0)
    gp(L.G_TIME_ISY, 5.8)
    gp(L.G_TIME_ISEV, 9.5)
    gp(L.G_TIME_ICRI, 7.1)
    gp(L.G_TRANSMISSION_PROB, 0.05)
    gp(L.G_REL_TRANSMISSION_NS, 0.7)
    gp(L.G_RECOVERED_PER_INS, 0.09)
    gp(L.G_RISK_FROM_SYMPTOMATIC, 0.25)
    gp(L.G_MAX_RISK_FROM_SYMPTOMATIC, 0.45)
    gp(L.G_SEVERE_PER_ISY, 0.2)
    gp(L.G_CRITICAL_PER_SEVERE, critical_per_severe)
    gp(L.G_DEATHS_PER_SEVERE, 0.0)
    gp(L.G_DEATHS_PER_CRITICAL, 0.3)

    y = np.zeros((G, 10))
    for g in range(G):
        y[g, L.E] = fact * 100
        y[g, L.INS] = fact * 50
        y[g, L.ISY] = fact * 50
        y[g, L.ISEV] = fact * 20
        y[g, L.ICRI] = fact * 10
        y[g, L.R] = fact * 10
        y[g, L.D] = fact * 0
        # Populations::set_difference_from_group_total (populations.h:194-205)
        cur = 0.0
        for c in range(10):
            cur += y[g, c]
        cur -= y[g, L.S]
        y[g, L.S] = fact * 10000 - cur

    base = np.full((1, 1, G, G), fact * 10.0)
    mini = np.zeros((1, 1, G, G))
    times, vals = L.damping_cache_single(G, 30.0, 0.7)
    return L.GraphArrays(G, p[None], base, mini, times[None, None], vals[None, None], y.reshape(1, -1),
                         np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, 10 * G)))


# name -> (csv, G, critical_per_severe, integrator opts, t0, tmax, dt, tolerance, summed over groups)
GOLDEN_CASES = {
    "py_osecir_ck54": ("ode-secihurd-compare.csv", 1, 0.25, dict(), 0.0, 50.0, 0.1, 1e-9),
    "py_osecir_ageres_ck54": ("ode-secihurd-ageres-compare.csv", 3, 0.25, dict(), 0.0, 50.0, 0.1, 1e-10),
    "cpp_ageres_ck54_bounded": ("secihurd-compare-cashkarp.csv", 3, 0.25,
                                dict(abs_tol=1e-1, rel_tol=1e-4, dt_min=0.3, dt_max=1.0), 0.0, 50.0, 0.3, 1e-10),
    "cpp_secir_rkf45": ("secihurd-compare.csv", 1, 0.3,
                        dict(method=L.METHOD_RKF45, abs_tol=1e-1, rel_tol=1e-3, dt_min=0.3, dt_max=1.0),
                        0.0, 50.0, 0.3, 1e-10),
    "cpp_ageres_rkf45": ("secihurd-compare.csv", 3, 0.3,
                         dict(method=L.METHOD_RKF45, abs_tol=1e-1, rel_tol=1e-4, dt_min=0.3, dt_max=1.0),
                         0.0, 50.0, 0.3, 1e-10),
}


def golden_case(name):
    csv, G, cps, opts, t0, tmax, dt, tol = GOLDEN_CASES[name]
    return dict(model=reference_test_model(G, cps), expected=load_csv(csv), G=G, opts=L.integrator_opts(**opts),
                t0=t0, tmax=tmax, dt=dt, tol=tol)


def sum_groups(values: np.ndarray, G: int) -> np.ndarray:
    """[P, 10G] -> [P, 10] summed over age groups."""
    return values.reshape(values.shape[0], G, 10).sum(axis=1)
