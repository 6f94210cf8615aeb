"""The 3D oracle pinned to the 2D TE oracle, and its own invariants (no GPU).

A 3D run that is invariant along a one-cell periodic axis is a 2D TE run in the other two:
(Ex, Ey, Hz) in the (x, y) plane, (Ey, Ez, Hx) in (y, z), (Ez, Ex, Hy) in (z, x). Each must
reproduce oracle/te_numpy.py — Etalon's update restated and pinned to Etalon's fixtures — bit
for bit: fields, psi and DFT accumulators, with CPML, a dielectric block and an E and an H
source. The three together fix every term of the six 3D updates. Then the two invariants of
Etalon's own unit tests (tests/unit/test_numpy_backend.py) in 3D: the discrete energy of a PEC
cavity and the exact mirror symmetries of a centred dipole.
"""

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from etalon_gb300 import yee3d
from oracle.yee3d_numpy import PSI, REDUCTIONS, Oracle3D, psi_name, to_2d
from tests.yee3d_cases import case3d, oracle_3d, oracle_te, reduced_oracle, roles, te_case


def raw(a):
    return np.ascontiguousarray(a).view(np.uint8)


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("red", REDUCTIONS, ids=["z-invariant", "x-invariant", "y-invariant"])
def test_invariant_run_is_the_2d_te_run(precision, red):
    p = te_case(precision)
    o2, o3 = oracle_te(p), reduced_oracle(p, red)
    o2.run(80)
    o3.run(80)
    mapped = roles(red)
    for name2d, name3d in mapped.items():
        assert np.array_equal(raw(to_2d(red, getattr(o3, name3d))), raw(getattr(o2, name2d))), (name2d, name3d)
    others = set(Oracle3D.FIELDS) - set(mapped.values())
    for name in others:
        assert not np.any(getattr(o3, name)), name
    for a2, a3 in zip(o2.acc, o3.acc):
        assert np.array_equal(raw(a2), raw(a3))
    assert np.abs(o2.hz).max() > 0 and np.abs(o2.psi_hz_x).max() > 0


def test_discrete_energy_is_conserved_in_a_pec_cavity():
    """W = ½Σε(Eⁿ)² + ½Σμ H^(n−½)·H^(n+½) is exactly invariant under the 3D leapfrog (PEC walls,
    anisotropic cells, a dielectric block), as Etalon's 2D test asserts for TE."""
    p = yee3d.yee3d_problem((0.8, 0.6, 0.5), (0.05, 0.04, 0.05), layers=0, background_eps=1.0,
                            boxes=[ph.Box((0.1, 0.0, 0.05), (0.3, 0.2, 0.2), 4.0)], precision="double")  # fmt: skip
    o = oracle_3d(p)
    rng = np.random.default_rng(3)
    for c in ("hx", "hy", "hz"):
        getattr(o, c)[...] = rng.standard_normal(getattr(o, c).shape)
    inv_cb = {c: 1.0 / getattr(o, "cb_" + c) for c in ("ex", "ey", "ez")}
    energies = []
    for _ in range(400):
        before = {c: getattr(o, c).copy() for c in ("hx", "hy", "hz")}
        o.update_h()
        w = sum(float((inv_cb[c] * getattr(o, c) ** 2).sum()) for c in ("ex", "ey", "ez"))
        w += sum(float((before[c] * getattr(o, c)).sum()) for c in ("hx", "hy", "hz")) / float(o.db)
        energies.append(w)
        o.update_e()
    assert np.abs(o.ex).max() > 0 and np.abs(o.ez).max() > 0
    np.testing.assert_allclose(energies, energies[0], rtol=1e-11)


def test_centred_dipole_gives_bitwise_symmetric_fields():
    """An Ez dipole on the centre node of a cube with CPML: mirror x, y and z and the swap x↔y
    hold exactly (E polar, H axial; mirroring z reverses the dipole)."""
    p = yee3d.yee3d_problem(
        (0.8, 0.8, 0.85), 0.05, layers=6, background_eps=2.085,
        sources=[ph.PointSource((0.0, 0.0, 0.0), "Ez", ph.GaussianPulse(1.55, 0.5))], precision="double",
    )  # fmt: skip
    assert p.injections[0].weights.size == 1
    o = oracle_3d(p)
    o.run(120)
    f = {c: getattr(o, c) for c in ("ex", "ey", "ez", "hx", "hy", "hz")}
    assert np.abs(f["ez"]).max() > 0 and np.abs(f["hx"]).max() > 0
    # parity under the mirror of axis a: E_c even unless c = a; H_c odd unless c = a
    for a in (0, 1):
        for c, v in f.items():
            odd = (c[1] == "xyz"[a]) if c[0] == "e" else (c[1] != "xyz"[a])
            m = np.flip(v, axis=a)
            np.testing.assert_array_equal(v, -m if odd else m, err_msg=f"{c} mirror {'xyz'[a]}")
    # mirror z reverses the z dipole: every sign above flips
    for c, v in f.items():
        odd = not ((c[1] == "z") if c[0] == "e" else (c[1] != "z"))
        m = np.flip(v, axis=2)
        np.testing.assert_array_equal(v, -m if odd else m, err_msg=f"{c} mirror z")
    t = (1, 0, 2)
    np.testing.assert_array_equal(f["ez"], f["ez"].transpose(t))
    np.testing.assert_array_equal(f["ex"], f["ey"].transpose(t))
    np.testing.assert_array_equal(f["hx"], -f["hy"].transpose(t))
    np.testing.assert_array_equal(f["hz"], -f["hz"].transpose(t))


def test_host_setup_of_an_invariant_run_matches_the_2d_setup():
    """yee3d_problem along the (x, y) plane with one periodic z cell and the 2D Δt casts the
    same cb and CPML profiles as te_problem (the 3D setup is the 2D one per axis)."""
    p2 = te_case("single")
    g2 = p2.grid
    p3 = yee3d.yee3d_problem((2.0, 1.5, 0.05), 0.05, layers=(8, 8, 0), periodic=(False, False, True),
                             background_eps=2.085, boxes=[ph.Box((0.1, -0.05, 0.0), (0.7, 0.35, 0.22), 11.7)],
                             dt=g2.dt, precision="single")  # fmt: skip
    assert p3.grid.n == (g2.nx, g2.ny, 1)
    c2, c3 = ph.cast_coefficients(p2), yee3d.cast_coefficients_3d(p3)
    assert np.array_equal(c3["cb_ex"][:, :, 0], c2.cb_ex) and np.array_equal(c3["cb_ey"][:, :, 0], c2.cb_ey)
    for k in ("b", "c", "ik"):
        for w in ("e", "h"):
            for a in ("x", "y"):
                assert np.array_equal(c3[f"{k}{a}_{w}"], getattr(c2, f"{k}{a}_{w}")), (k, a, w)
    assert c3["db"] == c2.db and c3["inv_dx"] == c2.inv_dx and c3["inv_dy"] == c2.inv_dy
    assert np.all(c3["bz_e"] == 1) and np.all(c3["cz_h"] == 0)


def test_layout_and_setup_errors():
    p = yee3d.yee3d_problem((0.4, 0.3, 0.2), 0.05, layers=(2, 3, 4))
    g = p.grid
    assert g.n == (12, 12, 12)
    assert g.shape("Ex") == (12, 13, 13) and g.shape("Hx") == (13, 12, 12) and g.shape("Hz") == (12, 12, 13)
    q = yee3d.yee3d_problem((0.4, 0.3, 0.2), 0.05, layers=2, periodic=(False, True, False))
    assert q.grid.n == (12, 6, 8) and q.grid.shape("Ex") == (12, 6, 9) and q.grid.pml_layers == (2, 0, 2)
    assert len(PSI) == 12 and len({psi_name(c, a) for c, a in PSI}) == 12
    # one periodic cell along z: sources and monitors take its single position
    r = case3d("single", periodic=(False, False, True), size=(1.2, 1.0, 0.05))
    assert r.grid.n[2] == 1 and [i.flat.size for i in r.injections] == [4, 2]
    with pytest.raises(ValueError, match="outside the grid"):
        yee3d.yee3d_problem((0.4, 0.3, 0.2), 0.05, layers=0,
                            sources=[ph.PointSource((5.0, 0.0, 0.0), "Ez", ph.GaussianPulse(1.55, 0.5))])  # fmt: skip


def test_trilinear_sampling_and_injection_weights():
    """Point sources and point monitors take the bracketing nodes along each axis with linear
    weights (etalon/fdtd/dft.py:39-66 per axis): the weights sum to one, a field linear in x, y
    and z interpolates exactly, and a plane monitor covers the nodes inside its span."""
    p = yee3d.yee3d_problem((1.0, 0.8, 0.6), 0.05, layers=4, background_eps=2.085,
                            sources=[ph.PointSource((0.013, -0.021, 0.037), "Ez", ph.GaussianPulse(1.55, 0.5))],
                            monitors=[ph.DFTMonitor("p", [1.55], center=(0.11, 0.07, -0.03)),
                                      ph.DFTMonitor("plane", [1.55], center=(0.0, 0.0, 0.0), size=(0.4, 0.3, 0.0),
                                                    components=("Hz",))])  # fmt: skip
    g = p.grid
    inj = p.injections[0]
    assert inj.flat.size == 8 and abs(inj.weights.sum() - 1.0) < 1e-12
    for s in p.samplings:
        x, y, z = g.coords(s.component)
        ii, jj, kk = np.unravel_index(s.flat_index, g.shape(s.component))
        if s.monitor == "p":
            f = 2.0 * x[ii] - 3.0 * y[jj] + 0.5 * z[kk] + 1.0  # linear: the interpolation is exact
            value = s.interpolate(f[None, :].astype(np.complex128))[0].real
            assert abs(value - (2.0 * 0.11 - 3.0 * 0.07 + 0.5 * -0.03 + 1.0)) < 1e-12
        else:
            assert np.all(np.abs(x[ii]) <= 0.2 + 1e-9) and np.all(np.abs(y[jj]) <= 0.15 + 1e-9)
            assert s.flat_index.size == np.unique(ii).size * np.unique(jj).size * np.unique(kk).size
    # the E coefficient of an injection uses the permittivity at each of its nodes
    i, j, k = np.unravel_index(inj.flat, g.shape("Ez"))
    expected = g.dt / (yee3d.EPSILON_0 * p.eps["Ez"][i, j, k]) * inj.weights / (g.dx * g.dy * g.dz * 1e-18)
    np.testing.assert_allclose(inj.coefficient, expected, rtol=1e-12)
