"""Comparison helpers for GPU-vs-oracle parity with readable first-mismatch reports."""
import numpy as np

# Control entries that are decisions or exact counters: must match exactly.
EXACT_CONTROL = {0: "accepted bank", 2: "accepted steps", 3: "rejections", 4: "pending", 5: "setup",
                 6: "converged", 7: "failure", 8: "iterations", 18: "total iterations", 21: "sweep",
                 29: "retries", 32: "trials", 33: "last rejection code", 57: "defect state",
                 58: "defect corrections", 61: "true residual converged", 88: "forcing min F",
                 89: "forcing max F", 20: "dt", 14: "max dt div", 15: "max speed", 16: "hydro error",
                 27: "max CFL"}


def first_mismatch(a, b, names=None):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return f"shape {a.shape} vs {b.shape}"
    bad = np.flatnonzero(~((a == b) | (np.isnan(a) & np.isnan(b))))
    if bad.size == 0:
        return None
    i = bad[0]
    return f"{bad.size} differ; first at {i}: {a[i]!r} vs {b[i]!r}" + (f" ({names(i)})" if names else "")


def bank_locator(n):
    nx, ny, nz = n
    N = nx * ny * nz
    NU = (nx + 1) * ny * nz
    NV = nx * (ny + 1) * nz
    NW = nx * ny * (nz + 1)

    def where(i):
        for name, base, dims in (("F", 0, (nx, ny, nz)), ("u", N, (nx + 1, ny, nz)), ("v", N + NU, (nx, ny + 1, nz)),
                                 ("w", N + NU + NV, (nx, ny, nz + 1)), ("p", N + NU + NV + NW, (nx, ny, nz))):
            size = dims[0] * dims[1] * dims[2]
            if base <= i < base + size:
                j = i - base
                return f"{name}[{j % dims[0]},{(j // dims[0]) % dims[1]},{j // (dims[0] * dims[1])}]"
        return "?"
    return where


def control_report(cg, co):
    out = []
    for k, name in EXACT_CONTROL.items():
        if not (cg[k] == co[k]):
            out.append(f"c[{k}] {name}: gpu {cg[k]!r} oracle {co[k]!r}")
    return out
