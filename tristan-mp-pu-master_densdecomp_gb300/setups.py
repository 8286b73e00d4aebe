"""Seeded synthetic initial conditions with the shapes of the reference's
problem setups.

The reference loads its plasma on the host through the user file
(user/user_weibel.F90:252-314: two counter-streaming beams, each injected by
inject_plasma_region with ppc0/2 per cell, code/particles.F90:2549-2938,
Maxwell-Juttner momenta from maxwell_dist, :2176-2273, then
reorder_particles). No dataset is involved; these loaders draw the same
shapes from numpy's PCG64 with a fixed seed:

* ion and electron of each pair share one position, uniform in the cell,
  so the initial charge density is exactly zero (as inject_plasma_region
  places both species of a pair at one point);
* momenta are an isotropic non-relativistic Maxwellian of temperature
  delgam (kT/mc^2) in the beam frame, Lorentz-boosted along +-x with the
  beam's gamma0 (gamma0 < 1 is read as v/c, code/particles.F90:208);
* pairs are laid out cell by cell in the reference's reorder key order
  (x fastest), beam -x before beam +x within a cell;
* ind counts up from 1 alternating ion / electron (inject_plasma_region's
  ``ind=++totalpartnum``), proc = 0, splitlev = 1, ch = 1.

The named workloads follow the reference's benchmark configurations: a
128x128 order-1 Weibel box (8 per cell per species), a 1024x1024 order-3
two-stream/Weibel box (16 per cell per species, beams at +-0.5c), a 256^3
order-2 Weibel box (4 per cell per species, gamma0 = 5), and an ensemble of
64 independent periodic 2D boxes whose sizes, plasmas and shape orders are
drawn from one seeded generator (ensemble_configs).
"""
from __future__ import annotations

import numpy as np

from .config import SimConfig

PARTICLE_DTYPE = np.dtype(
    [("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("u", "<f4"), ("v", "<f4"), ("w", "<f4"),
     ("ch", "<f4"), ("ind", "<i4"), ("proc", "<i4"), ("splitlev", "<i4")]
)

WORKLOADS = {
    # 2D Weibel, CPU-runnable: 128^2, order 1, 8 ppc/species, gamma0 = 3
    "weibel2d_128_o1": dict(dims=2, order=1, nx=128, ny=128, c=0.45, c_omp=10.0, ppc0=16.0,
                            gamma0=3.0, delgam=0.01, ntimes=4),
    # 2D two-stream/Weibel: 1024^2, order 3, 16 ppc/species, beams +-0.5c
    "twostream2d_1024_o3": dict(dims=2, order=3, nx=1024, ny=1024, c=0.45, c_omp=10.0,
                                ppc0=32.0, gamma0=0.5, delgam=0.005, ntimes=4),
    # the same plasma on a 512^2 box (8.4 M particles, 370 MB of particle
    # data: still above L2) for kernel profiling
    "twostream2d_512_o3": dict(dims=2, order=3, nx=512, ny=512, c=0.45, c_omp=10.0,
                               ppc0=32.0, gamma0=0.5, delgam=0.005, ntimes=4),
    # 2D pair shock: 8192 x 512, order 3, 16 ppc/species (ppc0 = 32),
    # gamma0 = 15, kT = 1e-4, sigma = 0.1, open x, reflecting wall, moving
    # injector (shock_params)
    "shock2d_8192x512_o3": dict(dims=2, order=3, nx=8192, ny=512, c=0.45, c_omp=10.0, ppc0=32.0,
                                gamma0=15.0, delgam=1e-4, sigma=0.1, ntimes=4, corr=1.0,
                                periodic=(0, 1, 1)),
    # 3D Weibel: 256^3, order 2, 4 ppc/species, gamma0 = 5
    "weibel3d_256_o2": dict(dims=3, order=2, nx=256, ny=256, nz=256, c=0.45, c_omp=8.0,
                            ppc0=8.0, gamma0=5.0, delgam=0.01, ntimes=4),
    # the same plasma on a 128^3 box (16.8 M particles, 740 MB of particle
    # data: still above L2) for kernel profiling
    "weibel3d_128_o2": dict(dims=3, order=2, nx=128, ny=128, nz=128, c=0.45, c_omp=8.0,
                            ppc0=8.0, gamma0=5.0, delgam=0.01, ntimes=4),
}


def make_config(name: str, **overrides) -> SimConfig:
    kw = dict(WORKLOADS[name])
    kw.update(overrides)
    return SimConfig(**kw)


def load_beams(cfg: SimConfig, seed: int = 123457, ppc_species: int | None = None):
    """Two counter-streaming pair beams filling the periodic interior.

    Returns (ions, lecs) as structured arrays with the reference's particle
    record. ``ppc_species`` defaults to ppc0/2 (both beams together).
    """
    rng = np.random.default_rng(seed)
    nps = int(round(cfg.ppc0 / 2)) if ppc_species is None else int(ppc_species)
    per_beam = max(nps // 2, 1)
    ng, ngz = cfg.nghost, cfg.nghostz
    x0 = ng // 2 + 1
    nx, ny = cfg.nx, cfg.ny
    nz = cfg.nz if cfg.dims == 3 else 1
    ncell = nx * ny * nz
    npairs = ncell * per_beam * 2
    # cell origins in reorder-key order (x fastest), beam -x then +x per cell
    cidx = np.repeat(np.arange(ncell, dtype=np.int64), per_beam * 2)
    beam = np.tile(np.repeat(np.array([-1.0, 1.0]), per_beam), ncell)
    ci = cidx % nx
    cj = (cidx // nx) % ny
    ck = cidx // (nx * ny)
    pos = np.empty((npairs, 3), np.float32)
    r = rng.random((npairs, 3), dtype=np.float32)
    # keep offsets strictly below 1 after rounding to float32
    r = np.minimum(r, np.float32(1.0 - 2.0 ** -24))
    pos[:, 0] = (ci + x0).astype(np.float32) + r[:, 0]
    pos[:, 1] = (cj + x0).astype(np.float32) + r[:, 1]
    if cfg.dims == 3:
        pos[:, 2] = (ck + (ngz // 2 + 1)).astype(np.float32) + r[:, 2]
    else:
        pos[:, 2] = np.float32(ngz // 2 + 1) + r[:, 2]
    g0 = cfg.gamma_drift
    beta0 = np.sqrt(1.0 - 1.0 / (g0 * g0))

    def momenta(delgam):
        th = rng.standard_normal((npairs, 3)) * np.sqrt(delgam)
        gam_rest = np.sqrt(1.0 + (th * th).sum(axis=1))
        ux = g0 * (th[:, 0] + beam * beta0 * gam_rest)
        return np.stack([ux, th[:, 1], th[:, 2]], axis=1).astype(np.float32)

    ui = momenta(cfg.delgam)
    ue = momenta(cfg.delgam * cfg.mi / cfg.me)
    ions = np.zeros(npairs, PARTICLE_DTYPE)
    lecs = np.zeros(npairs, PARTICLE_DTYPE)
    for arr, u in ((ions, ui), (lecs, ue)):
        arr["x"], arr["y"], arr["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
        arr["u"], arr["v"], arr["w"] = u[:, 0], u[:, 1], u[:, 2]
        arr["ch"] = 1.0
        arr["proc"] = 0
        arr["splitlev"] = 1
    ids = np.arange(npairs, dtype=np.int64)
    ions["ind"] = (2 * ids + 1).astype(np.int32)
    lecs["ind"] = (2 * ids + 2).astype(np.int32)
    return ions, lecs


def with_capacity(cfg: SimConfig, nions: int, nlecs: int) -> SimConfig:
    if cfg.maxhlf == 0:
        cfg.maxhlf = int(max(nions, nlecs) * 1.25) + 1024
    return cfg


ENSEMBLE_SIDES = (128, 192, 256, 384, 512)


def ensemble_configs(nbox: int = 64, seed: int = 20240607, sides=ENSEMBLE_SIDES, ppc_range=(4, 32),
                     fixed: bool = True, **overrides):
    """Per-box configurations of a seeded ensemble of periodic 2D boxes:
    each side uniform on `sides`, particles per cell per species uniform on
    the even numbers of `ppc_range` (two equal beams), beam gamma0 uniform on
    [1.5, 10], kT/mc^2 log-uniform on [1e-3, 1e-1], shape order uniform on
    {1, 2, 3}; c = 0.45, c_omp = 10, ntimes = 4. Returns (configs, table),
    the table listing the draws per box."""
    rng = np.random.default_rng(seed)
    cfgs, table = [], []
    for b in range(nbox):
        nx = int(rng.choice(sides))
        ny = int(rng.choice(sides))
        nps = 2 * int(rng.integers(ppc_range[0] // 2, ppc_range[1] // 2 + 1))
        gamma0 = float(rng.uniform(1.5, 10.0))
        delgam = float(10.0 ** rng.uniform(-3.0, -1.0))
        order = int(rng.integers(1, 4))
        kw = dict(dims=2, order=order, nx=nx, ny=ny, c=0.45, c_omp=10.0, ppc0=float(2 * nps),
                  gamma0=gamma0, delgam=delgam, ntimes=4, fixed=int(fixed))
        kw.update(overrides)
        cfgs.append(SimConfig(**kw))
        table.append(dict(box=b, nx=nx, ny=ny, ppc_species=nps, gamma0=gamma0, delgam=delgam, order=order))
    return cfgs, table


def load_ensemble(cfgs, seed: int = 123457):
    """Beams of every box (box b drawn with seed + b); sets each maxhlf."""
    out = []
    for b, cfg in enumerate(cfgs):
        ions, lecs = load_beams(cfg, seed=seed + b)
        with_capacity(cfg, len(ions), len(lecs))
        out.append((ions, lecs))
    return out


def shock_params(cfg: SimConfig, betainj: float = 0.99999, leftwall: float = 20.0, btheta: float = 90.0,
                 bphi: float = 0.0, wallgam: float = 1.0, temperature_ratio: float = 1.0,
                 dseed: float = 123457.0):
    """Hooks and initial fields of the collisionless-shock setup
    (user_pu/user_shock_pu.F90 with wall = 1, rightclean = 0,
    rightwall = 0), evaluated in single precision in the reference's order:
    read_input_user (:118-186: wallgam, betainj, pcosthmult), init_EMfields
    (:224-262: Binit, B along (btheta, bphi), E = -v x B of the upstream
    flow), init_particle_distribution_user (:271-330: wall and injector
    positions, x1in = 3, x2in = mx0 - 2), field_bc_user (:460-488).
    Sets cfg.window; returns (hooks dict, initial fields dict, initial-load
    region (x1, x2, y1, y2, ppc, weight))."""
    f32 = np.float32
    c = f32(cfg.c)
    g0 = f32(cfg.gamma0)
    if g0 < 1:
        g0 = f32(np.sqrt(f32(1.0) / (f32(1.0) - g0 * g0)))
    beta = f32(np.sqrt(f32(1.0) - f32(1.0) / (g0 * g0)))
    qi = f32(cfg.qi)
    me = f32(cfg.me) * abs(qi)
    mi = f32(cfg.mi) * abs(qi)
    ppc0 = f32(cfg.ppc0)
    binit = f32(np.sqrt(f32(f32(f32(f32(g0 * ppc0) * f32(0.5)) * f32(c * c)) * f32(me * f32(f32(1.0) + me / mi)))
                        * f32(cfg.sigma)))
    pi_d = float(np.float32(3.1415927))
    bth = f32(float(f32(btheta) / f32(180.0)) * pi_d)
    bph = f32(float(f32(bphi) / f32(180.0)) * pi_d)
    cos_t, sin_t = f32(np.cos(float(bth))), f32(np.sin(float(bth)))
    cos_p, sin_p = f32(np.cos(float(bph))), f32(np.sin(float(bph)))
    bx0 = f32(binit * cos_t)
    by0 = f32(f32(binit * sin_t) * sin_p)
    bz0 = f32(f32(binit * sin_t) * cos_p)
    ex0 = f32(0.0)
    ey0 = f32((-beta) * bz0)
    ez0 = f32(-((-beta) * by0))
    wg = f32(wallgam)
    if wg == 0:
        wg = f32(1.0)
    if wg < 1:
        wg = f32(np.copysign(f32(1.0) / np.sqrt(f32(1.0) - wg * wg), wg))
    betawall = f32(np.sqrt(f32(1.0) - f32(1.0) / (wg * wg)))
    mx, my = cfg.mx, cfg.my
    xinject2 = float(f32(f32(mx - 2.0) / f32(2.0)))
    delgam_i = f32(cfg.delgam)
    delgam_e = f32(f32(f32(delgam_i * mi) / me) * f32(temperature_ratio))
    sh = dict(wall=1, walloc=float(leftwall), gammawall=float(wg), betawall=float(betawall),
              cond_i1=1, cond_i2=int(leftwall - 5.0), edge_i1=mx - 2, edge_i2=mx,
              edge=[float(v) for v in (ex0, ey0, ez0, bx0, by0, bz0)],
              inject=1, xinject2=xinject2, betainj=float(f32(betainj)), xinj_max=float(mx - 15),
              ppc0=float(ppc0), gamma_drift=float(-g0), weight=1.0, y1=3.0, y2=float(my - 2.0),
              delgam_i=float(delgam_i), delgam_e=float(delgam_e),
              pcosthmult=1.0 if binit != 0 else 0.0, sigma_nonzero=int(cfg.sigma != 0),
              dseed=float(dseed), totalpartnum=0)
    n = cfg.ncells
    fields = {k: np.full(n, v, np.float32) for k, v in
              (("ex", ex0), ("ey", ey0), ("ez", ez0), ("bx", bx0), ("by", by0), ("bz", bz0))}
    cfg.window = (3.0, float(mx - 2.0)) + tuple(cfg.window_in()[2:]) if cfg.window is None else cfg.window
    region = (float(f32(leftwall)), float(f32(xinject2)), 3.0, float(my - 2.0), float(ppc0), 1.0)
    return sh, fields, region


def shock_capacity(cfg: SimConfig, laps: int, sh: dict) -> int:
    """particles per species after the initial load and `laps` injections"""
    per_lap = 0.5 * cfg.ppc0 * (cfg.my - cfg.nghost) * (1.0 + sh["betainj"]) * cfg.c
    init = 0.5 * cfg.ppc0 * (cfg.my - cfg.nghost) * (sh["xinject2"] - 20.0)
    return int(init + per_lap * (laps + 2)) + 4096
