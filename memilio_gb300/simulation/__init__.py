"""Python entry mirroring MEmilio's `memilio.simulation` module
(pycode/memilio-simulation, bindings in cpp/.../bindings) for the ODE-SECIR
path, over libmiogpu's C ABI (ctypes, `memilio_gb300._native`).

    import memilio_gb300.simulation as mio
    import memilio_gb300.simulation.osecir as osecir

replaces

    import memilio.simulation as mio
    import memilio.simulation.osecir as osecir

for the classes used with the ODE-SECIR model: AgeGroup, Damping,
MobilityParameters, TimeSeries results and interpolate_simulation_result.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from .. import layout as L


class AgeGroup(int):
    """mio.AgeGroup: an index into the age groups."""


@dataclass
class Damping:
    """mio.Damping(coeffs, t, level=0, type=0): factors active from time t."""
    coeffs: np.ndarray
    t: float
    level: int = 0
    type: int = 0

    def __post_init__(self):
        self.coeffs = np.atleast_1d(np.asarray(self.coeffs, np.float64))
        self.t = float(self.t)


def damping_cache(shape, dampings: Sequence[Damping]):
    """Dampings::update_cache (memilio/epidemiology/damping.h:570-600): the
    accumulated damping matrices at each distinct damping time, in the order
    Dampings keeps them (by time, type, level; an equal key replaced): a new
    damping replaces the active one of its (level, type), matrices of one level
    add, levels combine as 1 - prod(1 - d). Returns (times [K], values [K, *shape])
    with K >= 2 (first point -DBL_MAX with zeros, last DBL_MAX)."""
    by_key = {}
    for d in dampings:  # an equal (time, type, level) replaces (Dampings::add_, :603-614)
        by_key[(d.t, d.type, d.level)] = d
    ordered = [by_key[k] for k in sorted(by_key)]
    times, values = [L.DBL_LOWEST], [np.zeros(shape)]
    active = []  # [level, type, matrix] in first-seen order (update_active_dampings, :616-658)
    sums = []    # [level, matrix] in first-seen order
    for d in ordered:
        m = np.broadcast_to(d.coeffs, shape).astype(np.float64)
        hit = next((a for a in active if a[0] == d.level and a[1] == d.type), None)
        lsum = next((x for x in sums if x[0] == d.level), None)
        if hit is not None:
            lsum[1] = lsum[1] + (m - hit[2])
            hit[2] = m
        else:
            active.append([d.level, d.type, m])
            if lsum is not None:
                lsum[1] = lsum[1] + m
            else:
                sums.append([d.level, m.copy()])
        comb = sums[0][1].copy()  # inclusive_exclusive_sum (:545-562)
        for _, other in sums[1:]:
            comb = comb + other - comb * other
        tb = times[-1]
        diff = abs(d.t - tb)
        if diff <= 1e-15 or diff <= 1e-15 * max(abs(d.t), abs(tb)):
            values[-1] = comb
        else:
            times.append(d.t)
            values.append(comb)
    times.append(L.DBL_MAX)
    values.append(values[-1])
    return np.array(times), np.array(values)


class MobilityParameters:
    """mio.MobilityParameters(coeffs): one coefficient per (age group, compartment)."""

    def __init__(self, coeffs):
        self.coeffs = np.asarray(coeffs, np.float64).ravel().copy()


class TimeSeries:
    """mio.TimeSeries: time points with one value vector each."""

    def __init__(self, num_elements: int):
        self._n = int(num_elements)
        self._t: List[float] = []
        self._v: List[np.ndarray] = []

    def add_time_point(self, t: float, v=None):
        self._t.append(float(t))
        self._v.append(np.zeros(self._n) if v is None else np.asarray(v, np.float64).copy())

    def get_num_time_points(self) -> int:
        return len(self._t)

    def get_num_elements(self) -> int:
        return self._n

    def get_time(self, i: int) -> float:
        return self._t[i]

    def get_last_time(self) -> float:
        return self._t[-1]

    def get_value(self, i: int) -> np.ndarray:
        return self._v[i]

    def get_last_value(self) -> np.ndarray:
        return self._v[-1]

    def __getitem__(self, i: int) -> np.ndarray:
        return self._v[i]

    def as_ndarray(self) -> np.ndarray:
        """[1 + num_elements, num_time_points]: the times, then the values."""
        if not self._t:
            return np.zeros((1 + self._n, 0))
        return np.vstack([np.array(self._t)[None, :], np.array(self._v).T])


def interpolate_simulation_result(ts: TimeSeries, abs_tol: float = 100 * 1e-12, times=None) -> TimeSeries:
    """interpolate_simulation_result (memilio/data/analyze_result.h:186-268): the
    values at whole days (or at `times`), linear between neighbouring points."""
    if times is None:
        day0 = int(math.ceil(ts.get_time(0) - abs_tol))
        day_max = int(math.floor(ts.get_last_time() + abs_tol))
        times = [float(d) for d in range(day0, day_max + 1)]
    out = TimeSeries(ts.get_num_elements())
    if not times or ts.get_num_time_points() == 0:
        return out
    k = 0
    if ts.get_time(0) >= times[0]:
        out.add_time_point(times[0], ts[0])
        k = 1
    i = 0
    while i + 1 < ts.get_num_time_points() and k < len(times):
        t0, t1 = ts.get_time(i), ts.get_time(i + 1)
        if t0 < times[k] <= t1:
            w = (times[k] - t0) / (t1 - t0)
            out.add_time_point(times[k], ts[i] + w * (ts[i + 1] - ts[i]))
            k += 1
        else:
            i += 1
    if k < len(times) and ts.get_last_time() < times[k]:
        out.add_time_point(times[k], ts.get_last_value())
    return out
