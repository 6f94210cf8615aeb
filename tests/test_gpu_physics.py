"""Etalon's M0 physics validations on this backend's resident engine (needs a GPU).

Etalon checks its 2D TE solver against analytic results in tests/validation/test_m0.py; V5
(late-time stability) and V6 (2D Green's function) are restated on TEEngine at their full
lengths with the same thresholds (setups in tests/m0_cases.py). The oracle passes the same
checks on the CPU (tests/test_oracle_physics.py).
"""

import numpy as np
import pytest

from etalon_gb300.engine import TEEngine
from etalon_gb300.solver import interpolate_monitor
from tests import m0_cases

pytestmark = pytest.mark.gpu


def test_v5_late_time_energy_decays_and_never_grows(gpu):
    """30 000 steps: the energy ends below 1e-8 of its peak and never grows after it."""
    p = m0_cases.late_time_problem()
    e = TEEngine(p)
    try:
        energy = m0_cases.late_time_energy(p, e.advance, lambda: (e.field("ex"), e.field("ey"), e.field("hz")))
    finally:
        e.close()
    peak = int(np.argmax(energy))
    assert energy[-1] < 1e-8
    assert np.all(np.diff(energy[peak:]) <= 1e-12)


@pytest.mark.parametrize("precision", ["single", "double"])
def test_v6_field_matches_2d_greens_function(gpu, precision):
    """Hz at r = 3 µm within 1 % of the analytic line-source field at 11 wavelengths."""
    pytest.importorskip("scipy.special")
    p, pulse, r = m0_cases.green_problem(precision)
    e = TEEngine(p)
    try:
        e.advance(p.n_steps)
        measured = interpolate_monitor(p.samplings[0], e.dft(0)).reshape(-1).astype(np.complex128)
    finally:
        e.close()
    ratio = measured / m0_cases.green_analytic(p, pulse, r)
    assert np.all(np.abs(ratio - 1.0) < 1e-2), ratio


@pytest.mark.parametrize("precision", ["single", "double"])
def test_v4_cpml_reflection_below_minus_80_db(gpu, precision):
    """Hz next to the CPML side and corner against a reflection-free larger box: within 1e-4
    of the reference's peak (Etalon's −80 dB guard; it measures about −91 dB)."""
    traces = []
    for p, idx in m0_cases.reflection_problems(precision=precision):
        e = TEEngine(p)
        try:
            traces.append(m0_cases.hz_traces(p, idx, e.advance, lambda: e.field("hz")))
        finally:
            e.close()
    assert np.abs(traces[1]).max() > 0
    assert np.all(m0_cases.reflection_error(*traces) < 1e-4)


def _gpu_dispersion(dl, n=1.0, precision="single"):
    p, probes = m0_cases.dispersion_problem(dl, n=n, precision=precision)
    e = TEEngine(p)
    try:
        e.advance(p.n_steps)
        accs = [e.dft(k) for k in range(len(p.samplings))]
    finally:
        e.close()

    def values(k):
        return interpolate_monitor(p.samplings[k], accs[k]).reshape(-1).astype(np.complex128)

    return m0_cases.dispersion_velocities(p, probes, values, n)


@pytest.mark.parametrize("precision", ["single", "double"])
def test_v1_v2_dispersion_and_phase_velocity(gpu, precision):
    """V1 (ṽp within 1e-3 of the Yee relation along 0° and 45°, anisotropy visible at 9 cells
    per wavelength) and V2 (resolved raw ṽp within 0.5 % of c), at Δ = 0.1 and 0.05 µm."""
    pytest.importorskip("scipy.optimize")
    cases = {dl: _gpu_dispersion(dl, precision=precision) for dl in (0.1, 0.05)}
    for dl, by_angle in cases.items():
        for angle, (cpw, v, v_yee) in by_angle.items():
            assert np.abs(v / v_yee - 1).max() < 1e-3, (dl, angle)
            assert np.all(np.abs(v[cpw >= 20] - 1) < 5e-3), (dl, angle)
    (cpw, axis, _), (_, diagonal, _) = cases[0.1][0.0], cases[0.1][45.0]
    coarsest = int(np.argmin(cpw))
    assert axis[coarsest] < 0.99 and diagonal[coarsest] - axis[coarsest] > 0.01


def test_v3_uniform_dielectric(gpu):
    pytest.importorskip("scipy.optimize")
    for angle, (_, v, v_yee) in _gpu_dispersion(0.05, n=1.5).items():
        assert np.abs(v / v_yee - 1).max() < 1e-3, angle
