"""2D TM mode on the GPU against the direct TM oracle, bit for bit (needs a GPU).

The engine steps a TM run as its dual TE run (etalon_gb300/tm.py) on the one-step and the
temporally blocked kernels with a per-node Ez coefficient (etg_sim_set_db_nodes; the blocked
tiles run their compile-time TM variant); oracle/tm_numpy.py writes the TM
update directly and is pinned to the TE oracle by tests/test_tm_oracle.py.
"""

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from etalon_gb300 import tm
from tests.test_tm_oracle import oracle_tm, raw, tm_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("steps", [160, 37])
@pytest.mark.parametrize(("kernel", "deep"), [("plain", False), ("tb", False), ("tb", True), ("tma", False)])
def test_tm_engine_matches_tm_oracle(gpu, precision, steps, kernel, deep):
    """One-step and temporally blocked kernels (default and deep tiles; a TMA-fed choice runs
    the plain blocked kernel), 37 steps ending in one-step remainders."""
    from etalon_gb300 import _lib

    boxes = [ph.Box((0.1, -0.05, 0.0), (0.7, 0.35, 0.22), 11.7)]
    p = tm_case(precision, boxes=boxes, background_eps=2.085, n_steps=160)
    o = oracle_tm(p)
    o.run(steps)
    with tm.TMEngine(p, kernel=kernel) as e:
        if deep:
            e.te.set_option(_lib.OPT_TB_DEPTH, 8 if precision == "single" else 4)
        e.advance(steps)
        e.synchronize()
        for name in o.FIELDS:
            assert np.array_equal(raw(e.field(name)), raw(getattr(o, name))), name
        for k in range(len(p.components)):
            assert np.array_equal(raw(e.dft(k)), raw(o.acc[k])), f"accumulator {k} ({p.components[k]})"
        res = e.result()
        assert set(res) == {"point", "plane"} and set(res["plane"]) == {"Ez", "Hy"}
        assert res["point"]["Ez"].shape == (2,)
    assert np.abs(o.ez).max() > 0 and np.abs(o.hx).max() > 0


def test_tm_runs_are_refused_by_batches_and_the_adjoint(gpu):
    import ctypes as C

    from etalon_gb300 import _lib

    p = tm_case("single", n_steps=8)
    with tm.TMEngine(p) as e:
        h = C.c_void_p()
        with pytest.raises(ValueError, match="TM mode"):
            _lib.call("etg_batch_create", C.byref(h), 1, (C.c_void_p * 1)(e.te._h.value))
        with pytest.raises(ValueError, match="TM mode"):
            _lib.call("etg_adj_create", C.byref(h), e.te._h, 20, 4, 20, 4)


def test_tm_column_segments_vs_tm_oracle(gpu):
    """The headline grid in TM mode (2024², the strip, an Ez source) with 40-row tiles and K = 8:
    the lean interior tiles run as column segments of the TM variant. 80 steps against the TM
    oracle, bit for bit (the wave has reached the segments above and below the source tile)."""
    import ctypes as C

    from etalon_gb300 import _lib
    from tests import cases

    p = tm.tm_problem(
        size=(40.0, 40.0), dl=0.02, background_eps=cases.EPS_OXIDE,
        boxes=[ph.Box((0.0, 0.0, 0.0), (42.0, 0.5, 0.22), cases.EPS_SILICON)], pml=ph.PMLSpec(layers=12),
        sources=[tm.TMPointSource((-15.0, 0.0, 0.0), ph.GaussianPulse(1.55, 0.5))],
        monitors=[ph.DFTMonitor("m", [1.5, 1.6], center=(5.0, 0.0, 0.0))], n_steps=80, precision="single",
    )  # fmt: skip
    o = oracle_tm(p)
    o.run(80)
    with tm.TMEngine(p) as e:
        e.te.set_option(_lib.OPT_TB_DEPTH, 8)
        e.advance(80)
        e.synchronize()
        used = C.c_int64()
        _lib.call("etg_sim_get_option", e.te._h, _lib.OPT_TB_SEGMENTS_USED, C.byref(used))
        assert used.value > 0
        for name in o.FIELDS:
            assert np.array_equal(raw(e.field(name)), raw(getattr(o, name))), name
        for k in range(len(p.components)):
            assert np.array_equal(raw(e.dft(k)), raw(o.acc[k])), k
