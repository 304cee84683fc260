"""Small seeded configurations shared by the parity tests (sizes the oracle finishes in seconds)."""
import waves_gb300 as wg


def tank_small(**kw):
    """Wall-variant sloshing tank, 24x16x8, sine surface, CG tol 1e-6."""
    return wg.config("tank", n=(24, 16, 8), **kw)


def tank_ref_cfl(**kw):
    """The same tank at the reference's hard-coded CFL 0.45 and tolerance 1e-4."""
    return wg.config("tank", n=(24, 16, 8), cfl=0.45, pressure_tolerance=1e-4, **kw)


def beach_coarse(**kw):
    """The beach geometry and forcing on a 62x24x8 grid (5x, 2x, 5x coarser)."""
    return wg.config("beach", n=(62, 24, 8), spacing=(0.125, 0.05, 0.25), **kw)


def beach_slope(**kw):
    """Beach spacing around the toe of the 1:6 slope, the whole grid inside the forcing zone."""
    return wg.config("beach", n=(64, 40, 8), origin=(0.5, -0.6, -0.2), **kw)


CASES = {"tank_small": tank_small, "tank_ref_cfl": tank_ref_cfl, "beach_coarse": beach_coarse,
         "beach_slope": beach_slope}
