"""Headless presentation (waves_render): the CUDA ray-march against the oracle's restatement of
water.gdshader / clay.gdshader on the same op-19 export, orthographic and perspective.

The traces (first entry, occupied length, first exit, queries) are FP32 with the shaders' operation
order on both sides and must agree bit for bit.  The colours add FP64 transcendentals (pow, exp,
sin, cos) rounded to FP32, which may differ in the last place between CUDA's and the host's
libraries: colours are held to 2e-6 absolute."""
import numpy as np
import pytest

import waves_gb300 as wg
from tests.cases import beach_slope, tank_small
from tests.compare import first_mismatch
from tests.oracle_ref import render as oracle_render

COLOUR_TOLERANCE = 2e-6


def camera(s, mode, ortho, width=192, height=108):
    """A view of the whole box from the front-right-top (the offset of presentation.gd's preset)."""
    cfg = s.cfg
    lo = np.array(cfg.origin[:], dtype=np.float64)
    ext = np.array(cfg.n[:], dtype=np.float64) * np.array(cfg.spacing[:], dtype=np.float64)
    centre = lo + 0.5 * ext
    eye = centre + np.array([1.5, 2.0, 3.0]) * (0.6 * ext.max())
    return s.render_params(width, height, mode=mode, orthographic=ortho, target=centre, eye=eye,
                           size=1.3 * ext.max(), fov_y_deg=40.0)


def check(s, p):
    img, tr = s.render(p, trace=True)
    planes, kinds = s.export_surface()
    ref_img, ref_tr = oracle_render(planes, kinds, s.cfg, p, np.float32(s.control()[1]))
    m = first_mismatch(tr.ravel(), ref_tr.ravel())
    assert not m, f"trace: {m}"
    err = np.abs(img - ref_img).max()
    assert err <= COLOUR_TOLERANCE, err
    hits = int((tr[..., 0] >= 0).sum())
    return img, tr, hits


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["beach_slope", "tank_small"])
def test_render_matches_oracle(gpu_lib, case):
    cfg = {"beach_slope": beach_slope, "tank_small": tank_small}[case]()
    s = wg.WavesSolver(cfg)
    s.request_steps(3)
    s.run()
    for mode in (0, 1):
        for ortho in (1, 0):
            img, tr, hits = check(s, camera(s, mode, ortho))
            assert hits > 0.05 * tr.shape[0] * tr.shape[1], (mode, ortho, hits)
            assert np.isfinite(img).all()
    s.close()


@pytest.mark.gpu
def test_render_device_buffers_and_clock(gpu_lib):
    """The device entry point writes the same image; the ripple phase follows the surface clock
    (clock_ready) and nothing else."""
    import torch
    s = wg.WavesSolver(beach_slope())
    s.request_steps(2)
    s.run()
    p = camera(s, 1, 1, 96, 64)
    img, tr = s.render(p, trace=True)
    rgba = torch.empty((p.height, p.width, 4), dtype=torch.float32, device="cuda")
    trace = torch.empty_like(rgba)
    torch.cuda.synchronize()
    s.render_device(p, rgba.data_ptr(), trace.data_ptr())
    s.synchronize()
    assert np.array_equal(rgba.cpu().numpy(), img) and np.array_equal(trace.cpu().numpy(), tr)
    p.clock_ready = 0
    img0, tr0 = s.render(p, trace=True)
    assert np.array_equal(tr0, tr)
    wet = tr[..., 0] >= 0
    assert wet.any() and not np.array_equal(img0[wet], img[wet])
    assert np.array_equal(img0[~wet], img[~wet])
    s.close()


@pytest.mark.gpu
def test_render_rejects_bad_parameters(gpu_lib):
    s = wg.WavesSolver(tank_small())
    for bad in ({"width": 0}, {"mode": 2}, {"size": 0.0}, {"eye": (0.0, 0.0, 0.0), "target": (0.0, 0.0, 0.0)}):
        p = s.render_params(32, 16)
        for k, v in bad.items():
            if isinstance(v, tuple):
                getattr(p, k)[:] = v
            else:
                setattr(p, k, v)
        with pytest.raises(wg.WavesError):
            s.render(p)
    s.close()
