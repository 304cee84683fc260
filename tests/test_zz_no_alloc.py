"""waves_liquid_volume_noalloc: the volume reduction for hosts that cannot let the library allocate
device memory (engine-owned GPU buffers, no cudaMalloc inside a frame).  Its input and output are
the caller's device memory; its scratch is the library's fixed device array.  Checked against the
solver's own initial-volume reduction (waves_stats().initial_volume_m3) on two calls in a row.
This file is collected last so that a stop-at-first-failure run has already run everything else."""
import ctypes as C

import numpy as np
import pytest

import waves_gb300 as wg


@pytest.mark.gpu
def test_liquid_volume_noalloc_matches_solver_twice(gpu_lib):
    import torch
    cfg = wg.config("beach")
    s = wg.WavesSolver(cfg)
    v0 = s.stats()["initial_volume_m3"]
    nx, ny, nz = cfg.n
    F = torch.from_numpy(np.ascontiguousarray(s.bank(-1)[:s.N])).to("cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        st = gpu_lib.waves_liquid_volume_noalloc(C.c_void_p(F.data_ptr()), nx, ny, nz, cfg.spacing[0], cfg.spacing[1],
                                                 cfg.spacing[2], C.c_void_p(out.data_ptr()), None)
        torch.cuda.synchronize()
        assert st == 0
        assert abs(out.item() - v0) <= 1e-12 * abs(v0), (out.item(), v0)
    # beyond the fixed scratch: 2048 x 1024 x 2 cells > 2,097,152
    st = gpu_lib.waves_liquid_volume_noalloc(C.c_void_p(F.data_ptr()), 2048, 1024, 2, 0.1, 0.1, 0.1,
                                             C.c_void_p(out.data_ptr()), None)
    assert st == 1
    s.close()
