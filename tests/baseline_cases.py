"""The benchmark configurations' own plasmas, loaded as the reference's
Weibel setup loads them (test infrastructure: the loader is the oracle's).

user/user_weibel.F90:252-314 (init_particle_distribution_user) injects two
counter-streaming pair beams over the whole periodic interior with
inject_plasma_region (code/particles.F90:2549-2938): x from xinject =
nghost/2 + 1 to xinject2 = mx0 - nghost/2, y likewise, z from 3 to mz0 - 2
(clipped to the interior in 3D, one cell in 2D), ppc = ppc0/2 per beam,
gamma_drift = -gamma0 for the first beam and +gamma0 for the second (|g| < 1
is read as v/c), Maxwell-Juttner momenta of temperature delgam from
maxwell_dist (2D: pcosthmult = 0 without a magnetic field, momenta in the x-y
plane; 3D: isotropic), one Park-Miller stream seeded with dseed = 123457,
ind counting up over both beams; then reorder_particles sorts each species
by cell. Both the oracle and the CUDA path start from these arrays.
"""
from __future__ import annotations

import math

import numpy as np

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

F32 = np.float32


def beam_pairs(cfg: SimConfig) -> int:
    """pairs one inject_plasma_region call loads: ceiling((0.5 ppc) dz dy dx)
    in single precision, ppc = ppc0/2"""
    nz = cfg.nz if cfg.dims == 3 else 1
    numps = F32(F32(F32(F32(0.5) * F32(cfg.ppc0 / 2.0)) * F32(nz)) * F32(cfg.ny)) * F32(cfg.nx)
    return int(math.ceil(float(numps)))


def weibel_config(name: str, **overrides) -> SimConfig:
    cfg = setups.make_config(name, **overrides)
    if cfg.maxhlf == 0:
        cfg.maxhlf = 2 * beam_pairs(cfg) + 1024
    return cfg


def weibel_load(cfg: SimConfig, dseed: float = 123457.0):
    """(ions, lecs) of the reference's Weibel initial load for cfg, in the
    order reorder_particles leaves them"""
    o = oracle.OracleSim(cfg)
    ng, ngz = cfg.nghost, cfg.nghostz
    mx0, my0 = cfg.nx + ng, cfg.ny + ng
    mz0 = cfg.nz + ngz if cfg.dims == 3 else 1
    pcosthmult = 1.0 if cfg.dims == 3 else 0.0
    o.shock_init(dict(wall=0, walloc=0.0, gammawall=1.0, betawall=0.0, cond_i1=0, cond_i2=0, edge_i1=0,
                      edge_i2=0, edge=[0.0] * 6, inject=0, xinject2=0.0, betainj=0.0, xinj_max=0.0,
                      ppc0=float(cfg.ppc0), gamma_drift=-float(cfg.gamma0), weight=1.0, y1=0.0, y2=0.0,
                      delgam_i=float(cfg.delgam), delgam_e=float(F32(F32(cfg.delgam) * F32(cfg.mi)) / F32(cfg.me)),
                      pcosthmult=pcosthmult, sigma_nonzero=0, dseed=dseed, totalpartnum=0))
    x1, x2 = float(ng // 2 + 1), float(mx0 - ng // 2)
    y1, y2 = float(ng // 2 + 1), float(my0 - ng // 2)
    z1, z2 = 3.0, float(mz0 - 2)
    ppc = float(F32(cfg.ppc0) / F32(2.0))
    for gd in (-float(cfg.gamma0), float(cfg.gamma0)):
        o.shock.gamma_drift = gd
        o.inject_region3(x1, x2, y1, y2, z1, z2, ppc, 1.0)
        assert o.shock.injected >= 0, "capacity"
    o.call("to_reorder_particles_")
    ions, lecs = o.ions.copy(), o.lecs.copy()
    del o
    return ions, lecs


def oracle_sim(cfg: SimConfig, ions, lecs, openmp: bool = True):
    o = oracle.OracleSim(cfg, openmp=openmp)
    o.set_particles(ions, lecs)
    return o


def by_ind(p: np.ndarray) -> np.ndarray:
    return p[np.argsort(p["ind"], kind="stable")]
