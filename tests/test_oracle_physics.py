"""The oracle passes Etalon's M0 physics validations V5 and V6 (tests/validation/test_m0.py)
with Etalon's thresholds, on the CPU (a few seconds each)."""

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from etalon_gb300.solver import interpolate_monitor
from oracle.te_numpy import OracleMonitor, OracleSource, OracleTE
from tests import m0_cases


def _oracle(p):
    return OracleTE(
        p.grid.nx, p.grid.ny, p.grid.dt, vars(ph.cast_coefficients(p)), p.real,
        [OracleSource(i.component, i.i, i.j, i.coefficient, (i.pulse.wavelength, i.pulse.bandwidth, i.pulse.amplitude))
         for i in p.injections],
        [OracleMonitor(s.component, s.flat_index, s.frequencies) for s in p.samplings],
    )  # fmt: skip


def test_v5_oracle_late_time_energy_decays():
    p = m0_cases.late_time_problem()
    o = _oracle(p)
    energy = m0_cases.late_time_energy(p, o.run, lambda: (o.ex, o.ey, o.hz))
    peak = int(np.argmax(energy))
    assert energy[-1] < 1e-8
    assert np.all(np.diff(energy[peak:]) <= 1e-12)


def test_v6_oracle_matches_2d_greens_function():
    pytest.importorskip("scipy.special")
    p, pulse, r = m0_cases.green_problem("single")
    o = _oracle(p)
    o.run(p.n_steps)
    measured = interpolate_monitor(p.samplings[0], o.acc[0]).reshape(-1).astype(np.complex128)
    ratio = measured / m0_cases.green_analytic(p, pulse, r)
    assert np.all(np.abs(ratio - 1.0) < 1e-2), ratio


def test_v4_oracle_cpml_reflection_below_minus_80_db():
    traces = []
    for p, idx in m0_cases.reflection_problems():
        o = _oracle(p)
        traces.append(m0_cases.hz_traces(p, idx, o.run, lambda: o.hz))
    assert np.abs(traces[1]).max() > 0
    assert np.all(m0_cases.reflection_error(*traces) < 1e-4)


def _oracle_dispersion(dl, n=1.0):
    p, probes = m0_cases.dispersion_problem(dl, n=n)
    o = _oracle(p)
    o.run(p.n_steps)

    def values(k):
        return interpolate_monitor(p.samplings[k], o.acc[k]).reshape(-1).astype(np.complex128)

    return m0_cases.dispersion_velocities(p, probes, values, n)


@pytest.fixture(scope="module")
def oracle_vacuum():
    pytest.importorskip("scipy.optimize")
    return {dl: _oracle_dispersion(dl) for dl in (0.1, 0.05)}


def test_v1_oracle_dispersion_matches_yee_relation(oracle_vacuum):
    for dl, cases in oracle_vacuum.items():
        for angle, (_, v, v_yee) in cases.items():
            assert np.abs(v / v_yee - 1).max() < 1e-3, (dl, angle)


def test_v1_oracle_dispersion_anisotropy_is_resolved(oracle_vacuum):
    (cpw, axis, _), (_, diagonal, _) = oracle_vacuum[0.1][0.0], oracle_vacuum[0.1][45.0]
    coarsest = int(np.argmin(cpw))
    assert axis[coarsest] < 0.99 and diagonal[coarsest] - axis[coarsest] > 0.01


def test_v2_oracle_raw_phase_velocity_within_half_percent(oracle_vacuum):
    for dl, cases in oracle_vacuum.items():
        for angle, (cpw, v, _) in cases.items():
            assert np.all(np.abs(v[cpw >= 20] - 1) < 5e-3), (dl, angle)


def test_v3_oracle_uniform_dielectric():
    pytest.importorskip("scipy.optimize")
    for angle, (_, v, v_yee) in _oracle_dispersion(0.05, n=1.5).items():
        assert np.abs(v / v_yee - 1).max() < 1e-3, angle
