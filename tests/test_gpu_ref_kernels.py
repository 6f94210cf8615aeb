"""Etalon's own CUDA kernels on this GPU against this package's kernels (needs a GPU).

The reference's update_te.cu and dft.cu, compiled unchanged from its sources
(oracle/build_ref.py) and launched with its CuPy backend's shapes (oracle/ref_kernels.py), step
the same problems as the resident engine, with the same host tables; fields, ψ and
accumulators must agree bit for bit. This is also what the bench's reference-kernel timing
runs.
"""

import numpy as np
import pytest

from etalon_gb300.engine import TEEngine
from tests import cases
from tests.golden_io import FIELDS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize(("name", "steps"), [("config1", 2000), ("g4_full", 600)])
def test_reference_kernels_match_engine(gpu, name, steps, precision):
    from oracle import ref_kernels
    from tests.ref_kernel_run import RefRun

    if not ref_kernels.available(precision):
        pytest.fail("the reference kernel images are missing: run oracle/build_ref.py where Etalon's tree is")
    p = cases.CASES[name](precision=precision, n_steps=steps)
    k = ref_kernels.RefKernels(precision)
    run = RefRun(k, p, steps)
    for _ in range(steps):
        run.step()
    e = TEEngine(p)
    e.advance(steps)
    e.synchronize()
    try:
        for f in FIELDS:
            assert np.array_equal(run.field(f).view(np.uint8), e.field(f).view(np.uint8)), f
        for m in range(len(p.samplings)):
            assert np.array_equal(run.acc(m), e.dft(m)), f"accumulator {m}"
        assert np.abs(e.field("hz")).max() > 0
        assert k.launches >= 2 * steps
    finally:
        run.close()
        e.close()
        k.close()
