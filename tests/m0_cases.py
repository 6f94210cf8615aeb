"""Setups and analytic references of Etalon's M0 physics validations (tests/validation/test_m0.py,
etalon/validation/m0.py), shared by the oracle's CPU run and the GPU engine's run."""

from __future__ import annotations

import math

import numpy as np

from etalon_gb300 import physics as ph

GREEN_WAVELENGTHS = np.linspace(1.3, 1.8, 11)


def centred_size(half_width: float, dl: float) -> float:
    """A region with an odd number of cells, so the origin is an Hz node."""
    return (2 * math.ceil(half_width / dl) + 1) * dl


def late_time_problem(precision: str = "single") -> ph.TEProblem:
    """V5: a Gaussian Hz pulse at the centre of a 2 µm vacuum box, 12-layer CPML, 30 000 steps."""
    dl = 0.05
    size = centred_size(1.0, dl)
    return ph.te_problem(size=(size, size), dl=dl, pml=ph.PMLSpec(layers=12),
                         sources=[ph.PointSource((0.0, 0.0, 0.0), "Hz", ph.GaussianPulse(1.55, 0.5))],
                         n_steps=30_000, precision=precision)  # fmt: skip


def late_time_energy(p: ph.TEProblem, advance, fields) -> np.ndarray:
    """Total field energy per unit length after steps 1, 51, 101, … (``advance(k)`` runs k
    steps, ``fields()`` returns Ex, Ey, Hz), normalised to its peak."""
    area = (p.grid.dx * ph.UM) * (p.grid.dy * ph.UM)
    energy = []
    for k in range(p.n_steps // 50):
        advance(1 if k == 0 else 50)
        ex, ey, hz = fields()
        w = 0.5 * ph.EPSILON_0 * (np.sum(ex.astype(float) ** 2) + np.sum(ey.astype(float) ** 2))
        w += 0.5 * ph.MU_0 * np.sum(hz.astype(float) ** 2)
        energy.append(w * area)
    energy = np.asarray(energy)
    return energy / energy.max()


def green_problem(precision: str = "single", dl: float = 0.05, radius: float = 3.0):
    """V6: Hz line source at the origin, point monitor at (r, 0) with r = round(3/dl)·dl."""
    pulse = ph.GaussianPulse(1.55, 0.5, amplitude=1.0)
    size = centred_size(radius + 1.5, dl)
    m = round(radius / dl)
    p = ph.te_problem(size=(size, size), dl=dl, pml=ph.PMLSpec(layers=12),
                      sources=[ph.PointSource((0.0, 0.0, 0.0), "Hz", pulse)],
                      monitors=[ph.DFTMonitor("probe", list(GREEN_WAVELENGTHS), center=(m * dl, 0.0, 0.0),
                                              components=("Hz",))],
                      run_time=250e-15, precision=precision)  # fmt: skip
    return p, pulse, m * dl


def yee_wavenumber_along_x(wavelengths_um, grid) -> np.ndarray:
    """k̃ (1/m) of the 2D Yee scheme in vacuum along x: sin(k̃Δx/2)/Δx = sin(ωΔt/2)/(cΔt)
    (Taflove & Hagness, ch. 4), solved in closed form."""
    omega = 2.0 * np.pi * ph.C_0_SI / (np.asarray(wavelengths_um, dtype=np.float64) * ph.UM)
    dx, dt = grid.dx * ph.UM, grid.dt
    return 2.0 / dx * np.arcsin(dx * np.sin(omega * dt / 2.0) / (ph.C_0_SI * dt))


def green_analytic(p: ph.TEProblem, pulse: ph.GaussianPulse, r_um: float) -> np.ndarray:
    """−(ωε0/4) K̂(ω) H0⁽¹⁾(k̃ r) for M_z = K(t) δ²(r), time convention e^(−iωt); K̂ is the DFT of
    the injected samples K(nΔt) with the monitor's Δt."""
    from scipy.special import hankel1

    g = p.grid
    t = np.arange(p.n_steps) * g.dt
    omega = 2.0 * np.pi * ph.C_0 / GREEN_WAVELENGTHS
    k_hat = (ph.pulse_signal(pulse, t)[None, :] * np.exp(1j * omega[:, None] * t[None, :])).sum(1) * g.dt
    k_yee = yee_wavenumber_along_x(GREEN_WAVELENGTHS, g)
    return -(omega * ph.EPSILON_0 / 4.0) * k_hat * hankel1(0, k_yee * r_um * ph.UM)


def reflection_problems(layers: int = 12, run_time: float = 100e-15, precision: str = "single"):
    """V4 (Taflove & Hagness, ch. 7): Hz at probes 2 cells inside the region, next to the side
    and the corner of a 3.05 µm box, against a box large enough that its boundary reflections
    arrive after the run. Returns [(problem, [(i, j) per probe])] for the small and the large box."""
    dl = 0.05
    size = centred_size(1.5, dl)
    edge = size / 2.0
    probes = [(edge - 2.5 * dl, 0.0), (edge - 2.5 * dl, edge - 2.5 * dl)]  # side, corner
    margin = ph.C_0 * run_time / 2.0
    src = [ph.PointSource((0.0, 0.0, 0.0), "Hz", ph.GaussianPulse(1.55, 0.5))]
    out = []
    for region in (size, centred_size(1.5 + margin, dl)):
        p = ph.te_problem(size=(region, region), dl=dl, pml=ph.PMLSpec(layers=layers), sources=src,
                          run_time=run_time, precision=precision)  # fmt: skip
        x, y = p.grid.coords("Hz")
        out.append((p, [(int(np.argmin(np.abs(x - px))), int(np.argmin(np.abs(y - py)))) for px, py in probes]))
    return out


def hz_traces(p: ph.TEProblem, idx, advance, hz) -> np.ndarray:
    """Hz at the probe nodes after every step, (n_steps, n_probes)."""
    trace = np.empty((p.n_steps, len(idx)))
    for n in range(p.n_steps):
        advance(1)
        h = hz()
        trace[n] = [float(h[i, j]) for i, j in idx]
    return trace


def reflection_error(small: np.ndarray, reference: np.ndarray) -> np.ndarray:
    """max_t |Hz − Hz_ref| / max_t |Hz_ref| per probe."""
    return np.abs(small - reference).max(0) / np.abs(reference).max(0)


BROADBAND = ph.GaussianPulse(1.35, 0.9)
BROADBAND_WAVELENGTHS = np.linspace(0.9, 1.8, 19)


def dispersion_problem(dl: float, n: float = 1.0, run_time: float = 200e-15, r_near: float = 1.5,
                       r_far: float = 4.5, precision: str = "single"):
    """V1–V3: broadband Hz point source at an Hz node in a medium of index n; Hz point monitors
    on Hz nodes at two distances along 0° and along 45°. Returns the problem and, per angle,
    the monitor indices and the two distances (µm)."""
    m_axis = (round(r_near / dl), round(r_far / dl))
    m_diag = (round(r_near / (math.sqrt(2) * dl)), round(r_far / (math.sqrt(2) * dl)))
    points = {0.0: [(m * dl, 0.0, m * dl) for m in m_axis],
              45.0: [(m * dl, m * dl, math.sqrt(2) * m * dl) for m in m_diag]}  # fmt: skip
    monitors, probes = [], {}
    for angle, pts in points.items():
        probes[angle] = []
        for x, y, r in pts:
            probes[angle].append((len(monitors), r))
            monitors.append(ph.DFTMonitor(f"{angle:g}-{len(monitors)}", list(BROADBAND_WAVELENGTHS),
                                          center=(x, y, 0.0), components=("Hz",)))  # fmt: skip
    size = centred_size(r_far + 1.0, dl)
    p = ph.te_problem(size=(size, size), dl=dl, background_eps=n * n, pml=ph.PMLSpec(layers=12),
                      sources=[ph.PointSource((0.0, 0.0, 0.0), "Hz", BROADBAND)], monitors=monitors,
                      run_time=run_time, precision=precision)  # fmt: skip
    return p, probes


def yee_phase_velocity(wavelengths_um, grid, angle: float, n: float = 1.0) -> np.ndarray:
    """ṽp / (c/n) of the 2D Yee scheme along 0° or 45° on square cells (Taflove & Hagness,
    ch. 4), from the closed forms sin(k̃Δ/2) = Δ sin(ωΔt/2)/(vΔt) and, on the diagonal,
    sin(k̃Δ/(2√2)) = Δ sin(ωΔt/2)/(√2 vΔt)."""
    v = ph.C_0_SI / n
    omega = 2.0 * np.pi * ph.C_0_SI / (np.asarray(wavelengths_um, dtype=np.float64) * ph.UM)
    d, dt = grid.dx * ph.UM, grid.dt
    s = d * np.sin(omega * dt / 2.0) / (v * dt)
    k = 2.0 / d * np.arcsin(s) if angle == 0.0 else 2.0 * math.sqrt(2.0) / d * np.arcsin(s / math.sqrt(2.0))
    return omega / (k * v)


def measured_phase_velocity(near: np.ndarray, far: np.ndarray, r_near: float, r_far: float,
                            n: float = 1.0) -> np.ndarray:
    """ṽp / (c/n) from the phase of far/near (which cancels the source spectrum) matched to the
    outgoing cylindrical wave arg H0⁽¹⁾(k̃ r_far) − arg H0⁽¹⁾(k̃ r_near); the 2π ambiguity is
    resolved against the exact k = 2πn/λ and k̃ found by bracketed root finding."""
    from scipy.optimize import brentq
    from scipy.special import hankel1

    def model(k: float) -> float:
        corr = np.angle(hankel1(0, np.array([k * r_far, k * r_near])) * np.exp(-1j * np.array([k * r_far, k * r_near])))
        return k * (r_far - r_near) + float(corr[0] - corr[1])

    phase = np.angle(far / near)
    k_exact = 2.0 * np.pi * n / BROADBAND_WAVELENGTHS
    k_meas = np.empty_like(k_exact)
    for q, (k0, phi) in enumerate(zip(k_exact, phase)):
        target = phi + 2.0 * np.pi * round((model(k0) - phi) / (2.0 * np.pi))
        k_meas[q] = brentq(lambda k, t=target: model(k) - t, 0.7 * k0, 1.3 * k0, xtol=1e-14)
    return k_exact / k_meas


def dispersion_velocities(p: ph.TEProblem, probes: dict, point_values, n: float = 1.0) -> dict:
    """{angle: (cells per wavelength, measured ṽp, Yee ṽp)}; ``point_values(k)`` returns the
    interpolated DFT of monitor k (one complex value per wavelength)."""
    out = {}
    for angle, ((k_near, r_near), (k_far, r_far)) in probes.items():
        v = measured_phase_velocity(point_values(k_near), point_values(k_far), r_near, r_far, n)
        out[angle] = (BROADBAND_WAVELENGTHS / (n * p.grid.dx), v,
                      yee_phase_velocity(BROADBAND_WAVELENGTHS, p.grid, angle, n))  # fmt: skip
    return out
