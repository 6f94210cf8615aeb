"""The bounded stage waits of the TMA-fed kernels give up cleanly (needs a GPU).

Every wait of the TMA-fed kernels (``tma``: persistent CTAs, ``pipe``: one persistent CTA per
SM claiming tiles) for its shared-memory stage has an iteration limit. Here the limit of the
first attempt is set to zero tries (etg_debug_set_wait_tries), so real copies — which do
complete — are never seen in time (with a few tries they often are: the next tile is staged
during the current one): the wait must flag ETG_ERR_TIMEOUT, wait once more (bounded) for the
copy in flight, and its CTA must return, with no fault and no hang. The context stays
usable: with the default limit restored, the same engine then reproduces the one-step kernels'
run bit for bit.
"""

import pytest

from etalon_gb300 import _lib
from etalon_gb300.engine import TEEngine
from tests import cases
from tests.golden_io import FIELDS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["tma", "pipe"])
def test_stage_wait_times_out_and_the_gpu_stays_usable(gpu, kernel):
    import numpy as np

    # 2024² cells: both kernels have interior tiles, which the pipelined kernel stages by TMA
    # (its CPML tiles load themselves)
    p = cases.config2("single", n_steps=64)
    e = TEEngine(p, kernel=kernel)
    ref = TEEngine(p, kernel="plain")
    try:
        _lib.call("etg_debug_set_wait_tries", 0)
        try:
            e.advance(16)
            with pytest.raises(_lib.EtgError, match="bounded device-side wait gave up"):
                e.synchronize()
        finally:
            _lib.call("etg_debug_set_wait_tries", -1)
        e.synchronize()  # the flag was cleared when it was reported
        e.reset()
        e.advance(64)
        e.synchronize()
        ref.advance(64)
        ref.synchronize()
        for f in FIELDS:
            assert np.array_equal(e.field(f), ref.field(f)), f
        for k in range(len(e.monitors)):
            assert np.array_equal(e.dft(k), ref.dft(k))
    finally:
        e.close()
        ref.close()
