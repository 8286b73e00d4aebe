"""Physics known-answer cases shared by the oracle tests (CPU) and the GPU
tests: each builds its plasma, runs it through a runner and returns the
measured rate together with the theory's.

A runner is made by ``make(cfg, ions, lecs)`` and returns ``(step, field)``:
``step()`` advances one lap, ``field(name)`` returns the field's (mz, my,
mx) array after the lap."""
import math

import numpy as np

from tristan_gb300 import setups
from tristan_gb300.config import SimConfig


def _zero_crossing_rate(probe: np.ndarray) -> float:
    """angular frequency of a sampled oscillation from its zero crossings"""
    sgn = np.sign(probe)
    cross = np.nonzero(sgn[1:] != sgn[:-1])[0]
    t = [c0 + probe[c0] / (probe[c0] - probe[c0 + 1]) for c0 in cross]
    assert len(t) >= 5
    return math.pi / float(np.mean(np.diff(t)))


def _plane(a: np.ndarray, cfg) -> np.ndarray:
    """the (my, mx) plane of a field: 2D z-plane 0, 3D the mean over the
    interior z-planes"""
    if cfg.dims == 2:
        return a[0]
    z0 = cfg.nghostz // 2 + 1
    return a[z0 - 1: z0 - 1 + cfg.nz].mean(axis=0)


def plasma_oscillation(make, order: int, dims: int = 2):
    """Cold neutral pair plasma (ion and electron of each pair at one point,
    at rest); the electrons get u = 0.01 sin(kx). Returns (measured w,
    w_p = c/c_omp) from the zero crossings of E_x's Fourier mode over three
    periods (dt = 1, no filter). The charges of code/particles.F90:189-256
    give each species w_p^2 / 2 and both species move. 2D: box 64 x 8, 8 per
    cell per species; 3D: box 64 x 8 x 8, 2 per cell per species."""
    nx, ny = 64, 8
    if dims == 2:
        cfg = SimConfig(dims=2, order=order, nx=nx, ny=ny, c=0.45, c_omp=10.0, ppc0=16.0, gamma0=1.0,
                        delgam=0.0, ntimes=0)
    else:
        cfg = SimConfig(dims=3, order=order, nx=nx, ny=ny, nz=8, c=0.45, c_omp=10.0, ppc0=4.0, gamma0=1.0,
                        delgam=0.0, ntimes=0)
    ions, lecs = setups.load_beams(cfg, seed=3)
    setups.with_capacity(cfg, len(ions), len(lecs))
    x0 = cfg.nghost // 2 + 1
    kk = 2 * math.pi / nx
    lecs["u"] = (0.01 * np.sin(kk * (lecs["x"] - x0))).astype(np.float32)
    step, field = make(cfg, ions, lecs)
    # E_x sits half a cell right of its node
    xe = (np.arange(cfg.mx) + 1) + 0.5 - x0
    si, sj = slice(x0 - 1, x0 - 1 + nx), slice(x0 - 1, x0 - 1 + ny)
    basis = np.sin(kk * xe[si])
    wp = cfg.c / cfg.c_omp
    probe = []
    for _ in range(int(3.2 * 2 * math.pi / wp)):
        step()
        probe.append(float(np.dot(_plane(field("ex"), cfg)[sj, si].mean(axis=0), basis)))
    return _zero_crossing_rate(np.array(probe)), wp


def two_stream(make, order: int):
    """Two cold pair beams at +-0.5c in a box 64 x 8 (the electrostatic mode
    along x is the only fast one), seeded by a small electron velocity
    modulation. Returns (fitted growth rate of |E_x(k)| over the linear
    phase, the cold relativistic two-beam rate: 1 = a [1/(w - k v0)^2 +
    1/(w + k v0)^2], a = w_p^2 / (2 g0^3), w_p^2 = (c/c_omp)^2 g0)."""
    nx, ny = 64, 8
    cfg = SimConfig(dims=2, order=order, nx=nx, ny=ny, c=0.45, c_omp=10.0, ppc0=32.0, gamma0=0.5, delgam=0.0,
                    ntimes=0)
    ions, lecs = setups.load_beams(cfg, seed=5)
    setups.with_capacity(cfg, len(ions), len(lecs))
    x0 = cfg.nghost // 2 + 1
    kk = 2 * math.pi / nx
    lecs["u"] = (lecs["u"] + 1e-4 * np.sin(kk * (lecs["x"] - x0))).astype(np.float32)
    step, field = make(cfg, ions, lecs)
    xe = (np.arange(cfg.mx) + 1) + 0.5 - x0
    si, sj = slice(x0 - 1, x0 - 1 + nx), slice(x0 - 1, x0 - 1 + ny)
    bs, bc = np.sin(kk * xe[si]), np.cos(kk * xe[si])
    amp = []
    for _ in range(650):
        step()
        ex = _plane(field("ex"), cfg)[sj, si].mean(axis=0)
        amp.append(math.hypot(float(ex @ bs), float(ex @ bc)))
    amp = np.array(amp)
    assert amp[649] > 100 * amp[299]  # still growing, not saturated
    rate = float(np.polyfit(np.arange(300, 650), np.log(amp[300:650]), 1)[0])
    g0 = cfg.gamma_drift
    kv = kk * cfg.c * math.sqrt(1.0 - 1.0 / g0 ** 2)
    a = (cfg.c / cfg.c_omp) ** 2 * g0 / (2.0 * g0 ** 3)
    # (w^2 - kv^2)^2 = 2a (w^2 + kv^2), a quadratic in w^2
    w2 = np.roots([1.0, -(2.0 * kv ** 2 + 2.0 * a), kv ** 4 - 2.0 * a * kv ** 2])
    return rate, float(np.sqrt(w2.astype(complex)).imag.max())


def weibel(make, order: int, mode: int, dims: int = 2):
    """Cold pair beams at gamma0 = 3 along +-x in a box 8 x 64 (3D: 8 x 64
    x 8, 2 per cell per species); the filamentation mode k = 2 pi mode / 64
    along y is seeded by a small net electron current (ions and electrons
    of a cold pair move together, so one beam's electrons speed up where
    the other's slow down). Returns (fitted growth rate of |B_z(k)| over the
    linear phase, the cold relativistic filamentation rate: w^2 - k^2 c^2 -
    w_p^2 / g0^3 - w_p^2 b0^2 k^2 c^2 / (g0 w^2) = 0, E along the beams)."""
    nx, ny = 8, 64
    if dims == 2:
        cfg = SimConfig(dims=2, order=order, nx=nx, ny=ny, c=0.45, c_omp=10.0, ppc0=32.0, gamma0=3.0,
                        delgam=0.0, ntimes=0)
    else:
        cfg = SimConfig(dims=3, order=order, nx=nx, ny=ny, nz=8, c=0.45, c_omp=10.0, ppc0=4.0, gamma0=3.0,
                        delgam=0.0, ntimes=0)
    ions, lecs = setups.load_beams(cfg, seed=9)
    setups.with_capacity(cfg, len(ions), len(lecs))
    x0 = cfg.nghost // 2 + 1
    kk = 2 * math.pi * mode / ny
    lecs["u"] = (lecs["u"] + 1e-4 * np.abs(lecs["u"]) * np.sin(kk * (lecs["y"] - x0))).astype(np.float32)
    step, field = make(cfg, ions, lecs)
    ye = (np.arange(cfg.my) + 1) + 0.5 - x0
    si, sj = slice(x0 - 1, x0 - 1 + nx), slice(x0 - 1, x0 - 1 + ny)
    bs, bc = np.sin(kk * ye[sj]), np.cos(kk * ye[sj])
    amp = []
    for _ in range(250):
        step()
        bz = _plane(field("bz"), cfg)[sj, si].mean(axis=1)
        amp.append(math.hypot(float(bz @ bs), float(bz @ bc)))
    amp = np.array(amp)
    assert amp[249] > 100 * amp[100]
    rate = float(np.polyfit(np.arange(100, 250), np.log(amp[100:250]), 1)[0])
    g0 = cfg.gamma_drift
    b0 = math.sqrt(1.0 - 1.0 / g0 ** 2)
    c = cfg.c
    wp2 = (c / cfg.c_omp) ** 2 * g0
    bq = kk ** 2 * c ** 2 + wp2 / g0 ** 3
    cq = wp2 * b0 ** 2 * kk ** 2 * c ** 2 / g0
    return rate, math.sqrt((math.sqrt(bq * bq + 4.0 * cq) - bq) / 2.0)
