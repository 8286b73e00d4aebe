"""One small lap of the GPU hot path on cuda:0, checked against the oracle.

A 2D order-3 box of 48 x 32 cells with two counter-streaming pair beams
(4 per cell per species): one fixed-point lap must match the oracle bit for
bit (fields and particles), one FP32 lap within 1e-5 norm-wise relative
error (1e-4 of the maximum element-wise). Raises on any mismatch or if the CUDA library is unavailable.
"""
from __future__ import annotations

import numpy as np

from . import setups
from .config import SimConfig
from .gpu import GpuSim


def _case(fixed: int):
    import oracle  # the checker (test infrastructure)

    cfg = SimConfig(dims=2, order=3, nx=48, ny=32, c=0.45, c_omp=4.0, ppc0=8.0, gamma0=3.0, delgam=0.01,
                    ntimes=4, fixed=fixed)
    ions, lecs = setups.load_beams(cfg, seed=11)
    setups.with_capacity(cfg, len(ions), len(lecs))
    rng = np.random.default_rng(12)
    fields = {k: (rng.standard_normal(cfg.ncells) * 0.02).astype(np.float32)
              for k in ("ex", "ey", "ez", "bx", "by", "bz")}
    o = oracle.OracleSim(cfg)
    o.set_particles(ions, lecs)
    for k, v in fields.items():
        o.fields[k][:] = v
    g = GpuSim(cfg)
    try:
        g.set_fields(**fields)
        g.sync_from_host()
        g.set_particles(ions, lecs)
        g.step(1)
        o.step(1)
        g.sync_to_host()
        for k in ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz"):
            ref, got = o.fields[k], g.fields[k]
            if fixed:
                if not np.array_equal(ref, got):
                    raise AssertionError(f"smoke: {k} differs from the oracle (fixed point)")
            else:
                d = got.astype(np.float64) - ref
                rel = float(np.linalg.norm(d) / max(np.linalg.norm(ref), 1e-300))
                if rel > 1e-5 or float(np.abs(d).max()) > 1e-4 * max(float(np.abs(ref).max()), 1e-30):
                    raise AssertionError(f"smoke: {k} relative error {rel:.3e} above tolerance")
        a, b = np.sort(g.ions, order="ind"), np.sort(o.ions, order="ind")
        for k in ("x", "y", "z", "u", "v", "w"):
            if not np.array_equal(a[k], b[k]):
                raise AssertionError(f"smoke: ion {k} differs from the oracle")
    finally:
        g.close()


def run() -> None:
    _case(fixed=1)
    _case(fixed=0)
    print("smoke: ok")
