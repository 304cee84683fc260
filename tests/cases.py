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


def beach_slope_bf16(**kw):
    """beach_slope with the BF16 multigrid (storage and smoothing in BF16, FP32 arithmetic)."""
    return beach_slope(mg_precision=16, **kw)


def tank_bf16(**kw):
    return tank_small(mg_precision=16, **kw)


def tank_jacobi(**kw):
    """Jacobi smoothing, rebuild-every-trial maintenance: the other multigrid options."""
    return tank_small(mg_smoother=0, mg_smoothing=2, mg_maintenance=0, **kw)


def beach_coarse_jacobi(**kw):
    """The coarse beach with Jacobi smoothing (two sweeps) and rebuild-every-trial maintenance: the
    Jacobi path on a five-level plan (two levels between the finest and a shared-memory bottom)."""
    return beach_coarse(mg_smoother=0, mg_smoothing=2, mg_maintenance=0, **kw)


def tank_periodic(**kw):
    """The small tank, periodic in x (the periodic-x index, delta and transfer paths)."""
    return tank_small(periodic_x=1, **kw)


def dam_break(**kw):
    """Fixture 1: a water column released in the 24x16x8 tank (large free-surface motion)."""
    return wg.config("default", n=(24, 16, 8), shape=1, pressure_tolerance=1e-6, **kw)


def jets(**kw):
    """Fixture 4: two colliding 2 m/s jets (CFL limits, retries)."""
    return wg.config("default", n=(24, 16, 8), shape=4, pressure_tolerance=1e-6, **kw)


def wave_periodic(**kw):
    """Fixture 5: one second-order Stokes wavelength over a periodic 0.8 m channel."""
    import math
    k = 2.0 * math.pi / (32 * 0.025)
    omega = math.sqrt(9.81 * k * math.tanh(k * 0.45))
    return wg.config("default", n=(32, 16, 8), shape=5, periodic_x=1, wave=(0.03, k, omega, 0.45),
                     stokes_second=1, **kw)  # the reference's CG tolerance, 1e-4


def box_pool(**kw):
    """Fixture 2: a falling block over a shallow pool."""
    return wg.config("default", n=(24, 16, 8), shape=2, pressure_tolerance=1e-6, **kw)


def inflow(**kw):
    """Fixture 3: a 0.25 m/s current under the surface."""
    return wg.config("default", n=(24, 16, 8), shape=3, pressure_tolerance=1e-6, **kw)


def absorber(**kw):
    """Fixture 6: the coarse beach with the right-hand absorber."""
    return beach_coarse(shape=6, **kw)


def height_normals(**kw):
    """The corrugated tank with height-function normals (flag bit 0)."""
    return tank_small(height_normals=1, **kw)


def linear_air(**kw):
    """A steeper corrugation with the linear air extension."""
    return tank_small(linear_air=1, corrugation=0.1, **kw)


def max_face_cfl(**kw):
    """The dam break with the CFL rate taken as the maximum over axes."""
    return dam_break(max_face_cfl=1, **kw)


def plain_transport(**kw):
    """MacCormack without the trace cache and without valid-band advection (flag bits 1, 2 off)."""
    return tank_small(transport_cache=0, active_advection=0, corrugation=0.1, **kw)


def interior_fast(**kw):
    """MacCormack with the interior sampling fast path (flag bit 3)."""
    return tank_small(transport_interior=1, corrugation=0.1, **kw)


def tank_structure(**kw):
    """The structure-only multigrid maintenance policy (mode 1)."""
    return tank_small(mg_maintenance=1, **kw)


def cheb2(**kw):
    """Two Chebyshev sweeps per smoothing call."""
    return tank_small(mg_smoothing=2, **kw)


def aggr3(**kw):
    """Aggregation transfers from level 3 on."""
    return tank_small(mg_aggregate_from=3, **kw)


CASES = {"tank_small": tank_small, "tank_ref_cfl": tank_ref_cfl, "beach_coarse": beach_coarse,
         "beach_slope": beach_slope, "beach_coarse_jacobi": beach_coarse_jacobi, "beach_slope_bf16": beach_slope_bf16,
         "tank_bf16": tank_bf16,
         "tank_jacobi": tank_jacobi, "tank_periodic": tank_periodic, "dam_break": dam_break, "jets": jets,
         "wave_periodic": wave_periodic, "box_pool": box_pool, "inflow": inflow, "absorber": absorber,
         "height_normals": height_normals, "linear_air": linear_air, "max_face_cfl": max_face_cfl,
         "plain_transport": plain_transport, "interior_fast": interior_fast, "tank_structure": tank_structure,
         "cheb2": cheb2, "aggr3": aggr3}
