"""waves_liquid_volume_noalloc: the volume reduction for hosts that cannot let the library allocate
device memory (engine-owned GPU buffers, no cudaMalloc inside a frame).  Its input and output are
the caller's device memory; its scratch is the library's fixed device array.  Checked against the
solver's own initial-volume reduction (waves_stats().initial_volume_m3), bit for bit, on two calls
in a row; on a ragged size against an FP64 host sum; at exactly the largest accepted size; and
refused one block beyond it.  This file is collected last so that a stop-at-first-failure run has
already run everything else."""
import ctypes as C

import numpy as np
import pytest

import waves_gb300 as wg

MAX_CELLS = 2_097_152


def _volume(lib, F, n, h, out):
    import torch
    out.fill_(-1.0)
    torch.cuda.synchronize()
    st = lib.waves_liquid_volume_noalloc(C.c_void_p(F.data_ptr()), n[0], n[1], n[2], h[0], h[1], h[2],
                                         C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    return st, out.item()


@pytest.mark.gpu
def test_liquid_volume_noalloc_matches_solver_twice(gpu_lib):
    import torch
    cfg = wg.config("beach")
    s = wg.WavesSolver(cfg)
    v0 = s.stats()["initial_volume_m3"]
    n, h = tuple(cfg.n), tuple(cfg.spacing)
    F_host = np.ascontiguousarray(s.bank(-1)[:s.N])
    F = torch.from_numpy(F_host).to("cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        st, v = _volume(gpu_lib, F, n, h, out)
        assert st == 0
        assert v == v0, (v, v0)  # the solver's reduction order: equal bits
    # a ragged size (the first nx*ny*(nz-1) cells: not a multiple of the 256-cell block)
    ragged = (n[0], n[1], n[2] - 1)
    count = ragged[0] * ragged[1] * ragged[2]
    assert count % 256 != 0
    cell = float(np.float32(h[0])) * float(np.float32(h[1])) * float(np.float32(h[2]))
    want = float(np.sum(F_host[:count].astype(np.float64) * cell))
    st, v = _volume(gpu_lib, F, ragged, h, out)
    assert st == 0
    assert abs(v - want) <= 1e-12 * abs(want), (v, want)
    s.close()


@pytest.mark.gpu
def test_liquid_volume_noalloc_size_limit(gpu_lib):
    import torch
    rng = np.random.default_rng(7)
    F_host = rng.random(MAX_CELLS, dtype=np.float32)
    F = torch.from_numpy(F_host).to("cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    h = (0.025, 0.025, 0.05)
    cell = float(np.float32(h[0])) * float(np.float32(h[1])) * float(np.float32(h[2]))
    want = float(np.sum(F_host.astype(np.float64) * cell))
    # exactly the largest accepted size: 2048 x 1024 x 1 cells = 8192 blocks of 256
    st, v = _volume(gpu_lib, F, (2048, 1024, 1), h, out)
    assert st == 0
    assert abs(v - want) <= 1e-12 * abs(want), (v, want)
    # one block beyond it is refused before anything runs; the output slot is left alone
    st, v = _volume(gpu_lib, F, (2048, 1024 + 1, 1), h, out)
    assert st == 1 and v == -1.0
