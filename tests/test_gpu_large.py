"""The 620x96x160 beach (9,523,200 cells, 8 multigrid levels): the oracle cannot keep pace at this
size, so the GPU run is checked through properties that hold at any size -- every trial accepted
or retried without a halt, the FP64 volume ledger closing to rounding, F inside [0, 1]."""
import numpy as np
import pytest

import waves_gb300 as wg


def large_beach():
    return wg.config("beach", n=(620, 96, 160), spacing=(0.0125, 0.0125, 0.025), pressure_tolerance=1e-6)


@pytest.mark.gpu
def test_large_beach_steps(gpu_lib):
    cfg = large_beach()
    s = wg.WavesSolver(cfg)
    s.request_steps(4)
    assert s.run() == 0
    st = s.stats()
    assert st["accepted_steps"] == 4 and st["failure"] == 0
    c = s.control()
    volume = c[17]
    assert volume > 0
    # the ledger identity: accepted volume = initial volume + committed rounding/compression +
    # boundary fluxes, to FP64 rounding of the per-block sums
    assert abs(st["conservation_residual_m3"]) <= 1e-9 * volume, (st["conservation_residual_m3"], volume)
    F = s.bank()[: s.N]
    assert np.all(F >= 0.0) and np.all(F <= 1.0)
    s.close()
