"""3D Yee engine on the GPU against the 3D oracle, bit for bit (needs a GPU).

oracle/yee3d_numpy.py is pinned to the 2D TE oracle, and so to Etalon's outputs, by
tests/test_yee3d_oracle.py. Here the CUDA engine (etalon_gb300/csrc/etg_yee3d.cu, through the
etg_yee3d_* C ABI) must match it on every field, psi and DFT accumulator: CPML on all faces,
periodic axes, an invariant (2D) run, float32 and float64, step counts that end inside and
on a 32-step graph, the fused step (one kernel over two buffer sets, sources applied inside
it) and the two-kernel step. At a size too large for the oracle, a centred dipole must stay
exactly mirror symmetric.
"""

import ctypes as C

import numpy as np
import pytest

from etalon_gb300 import _lib
from etalon_gb300 import physics as ph
from etalon_gb300 import yee3d
from oracle.yee3d_numpy import Oracle3D
from tests.yee3d_cases import case3d, oracle_3d

pytestmark = pytest.mark.gpu


def raw(a):
    return np.ascontiguousarray(a).view(np.uint8)


CASES = {
    "cpml": dict(),
    "periodic-z": dict(periodic=(False, False, True), size=(1.2, 1.0, 0.3)),
    "periodic-xy": dict(periodic=(True, True, False), layers=5, size=(0.6, 0.5, 1.0)),
    "invariant-z": dict(periodic=(False, False, True), size=(1.2, 1.0, 0.05)),
}


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "two-kernel"])
@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("steps", [70, 32])
@pytest.mark.parametrize("case", list(CASES))
def test_engine_matches_oracle(gpu, precision, steps, case, fused):
    p = case3d(precision, n_steps=steps, **CASES[case])
    o = oracle_3d(p)
    o.run(steps)
    with yee3d.Yee3DEngine(p, fused=fused) as e:
        e.advance(steps)
        e.synchronize()
        assert e.n == steps
        for name in Oracle3D.FIELDS:
            assert np.array_equal(raw(e.field(name)), raw(getattr(o, name))), name
        for k in range(len(p.samplings)):
            assert np.array_equal(raw(e.dft(k)), raw(o.acc[k])), f"accumulator {k}"
    assert np.abs(o.ez).max() > 0 and np.abs(o.hy).max() > 0


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "two-kernel"])
@pytest.mark.parametrize("precision", ["single", "double"])
def test_engine_from_a_random_state(gpu, precision, fused):
    """Uploaded fields and psi (inside the strips) continue exactly as in the oracle."""
    p = case3d(precision, n_steps=40)
    o = oracle_3d(p)
    rng = np.random.default_rng(11)
    g = p.grid
    with yee3d.Yee3DEngine(p, fused=fused) as e:
        for c in ("ex", "ey", "ez", "hx", "hy", "hz"):
            v = rng.standard_normal(getattr(o, c).shape).astype(p.real)
            getattr(o, c)[...] = v
            e.set_field(c, v)
        # psi where the CPML of its axis is live (the leading strip of each profile)
        for name in Oracle3D.FIELDS[6:]:
            axis = "xyz".index(name[-1])
            v = np.zeros(getattr(o, name).shape, p.real)
            sl = [slice(None)] * 3
            sl[axis] = slice(0, g.pml_layers[axis])
            v[tuple(sl)] = rng.standard_normal(v[tuple(sl)].shape)
            getattr(o, name)[...] = v
            e.set_field(name, v)
        # the E arrays on PEC walls stay as uploaded; the oracle keeps them as well
        o.run(33)
        e.advance(33)
        e.synchronize()
        for name in Oracle3D.FIELDS:
            assert np.array_equal(raw(e.field(name)), raw(getattr(o, name))), name
        # switching the step form mid-run continues the same bits
        e.set_fused(not fused)
        o.run(7)
        e.advance(7)
        e.synchronize()
        for name in Oracle3D.FIELDS:
            assert np.array_equal(raw(e.field(name)), raw(getattr(o, name))), name


def test_large_centred_dipole_stays_symmetric(gpu):
    """160 x 160 x 161 cells with CPML, Ez dipole on the centre node, fp32, 300 steps: mirror x,
    y, z and the swap x↔y hold bit for bit (far past the oracle's sizes)."""
    p = yee3d.yee3d_problem((6.4, 6.4, 6.44), 0.04, layers=12, background_eps=2.085,
                            sources=[ph.PointSource((0.0, 0.0, 0.0), "Ez", ph.GaussianPulse(1.55, 0.5))],
                            n_steps=300, precision="single")  # fmt: skip
    assert p.injections[0].weights.size == 1
    with yee3d.Yee3DEngine(p) as e:
        e.advance(300)
        e.synchronize()
        f = e.fields()
    assert np.abs(f["Ez"]).max() > 0 and np.abs(f["Hx"]).max() > 0
    for a in (0, 1):
        for c, v in f.items():
            odd = (c[1] == "xyz"[a]) if c[0] == "E" else (c[1] != "xyz"[a])
            m = np.flip(v, axis=a)
            assert np.array_equal(v, -m if odd else m), f"{c} mirror {'xyz'[a]}"
    for c, v in f.items():
        odd = not ((c[1] == "z") if c[0] == "E" else (c[1] != "z"))
        m = np.flip(v, axis=2)
        assert np.array_equal(v, -m if odd else m), f"{c} mirror z"
    t = (1, 0, 2)
    assert np.array_equal(f["Ez"], f["Ez"].transpose(t)) and np.array_equal(f["Ex"], f["Ey"].transpose(t))
    assert np.array_equal(f["Hx"], -f["Hy"].transpose(t)) and np.array_equal(f["Hz"], -f["Hz"].transpose(t))


def test_engine_refusals(gpu):
    p = case3d("single", n_steps=10, periodic=(True, False, False), size=(0.3, 1.0, 0.8))
    with yee3d.Yee3DEngine(p) as e:
        with pytest.raises(RuntimeError, match="table covers steps"):
            e.advance(11)
        e.advance(10)
        e.synchronize()
        # psi of the periodic x axis is not stored: only zeros are accepted
        z = np.zeros(e.shape("psi_hz_x"), np.float32)
        e.set_field("psi_hz_x", z)
        assert not np.any(e.field("psi_hz_x"))
        with pytest.raises(RuntimeError, match="without CPML"):
            e.set_field("psi_hz_x", z + 1)
        h = C.c_void_p()
        with pytest.raises(ValueError, match="bad arguments"):
            _lib.call("etg_yee3d_create", C.byref(h), _lib.F32, 0, 4, 4, 0)
        flat = np.array([10**9], np.int64)
        table = np.zeros((4, 1), np.float32)
        with pytest.raises(ValueError, match="outside component"):
            _lib.call("etg_yee3d_add_source", e._h, 2, 1, flat.ctypes.data, 0, 4, table.ctypes.data)


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "two-kernel"])
@pytest.mark.parametrize("layout", ["duplicates", "many"])
def test_source_injection_semantics(gpu, fused, layout):
    """NumPy's field[nodes] -= delta, source by source: a node listed twice in one source keeps
    its last delta, two sources on one node subtract in turn; more source nodes than the fused
    kernel holds (32 per phase) run the two-kernel step. Against the oracle, bit for bit."""
    import dataclasses

    base = case3d("single", n_steps=40)
    ez, hy = base.injections
    if layout == "duplicates":
        twice = dataclasses.replace(ez, flat=np.concatenate([ez.flat, ez.flat[:2]]),
                                    weights=np.concatenate([ez.weights, ez.weights[:2]]),
                                    coefficient=np.concatenate([ez.coefficient, 3.0 * ez.coefficient[:2]]))  # fmt: skip
        injections = [twice, ez, hy, hy]
    else:
        injections = [dataclasses.replace(ez, coefficient=(1.0 + 0.25 * q) * ez.coefficient) for q in range(6)] + [hy]
    p = dataclasses.replace(base, injections=injections)
    o = oracle_3d(p)
    o.run(40)
    with yee3d.Yee3DEngine(p, fused=fused) as e:
        e.advance(40)
        e.synchronize()
        for name in Oracle3D.FIELDS:
            assert np.array_equal(raw(e.field(name)), raw(getattr(o, name))), name
        for k in range(len(p.samplings)):
            assert np.array_equal(raw(e.dft(k)), raw(o.acc[k])), f"accumulator {k}"
    assert sum(i.flat.size for i in injections if not i.is_magnetic) > (32 if layout == "many" else 0)
