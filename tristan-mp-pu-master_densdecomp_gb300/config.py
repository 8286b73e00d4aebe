"""Run configuration: the reference's `input` keys and the quantities the
reference derives from them at start-up.

Mirrors read_input_grid (code/fields.F90:154-192: ghost widths from the shape
order, full extents mx = mx0 + nghost), allocate_fields (code/fields.F90:
330-338: strides ix=1, iy=mx, iz=mx*my; 2D iz=0, mz=1), read_input_particles
(code/particles.F90:189-233: charge and mass normalisation, in single
precision), allocate_particles (code/particles.F90:286-341: maxhlf, the open
boundary window x1in..z2in) and read_input_algorithm
(code/initialize.F90:293-305: Corr, ntimes).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

f32 = np.float32


@dataclasses.dataclass
class SimConfig:
    dims: int = 2
    order: int = 1
    # interior cells per axis (the `input` file's mx0, my0, mz0)
    nx: int = 128
    ny: int = 128
    nz: int = 1
    c: float = 0.45
    c_omp: float = 10.0
    ppc0: float = 16.0
    gamma0: float = 3.0
    delgam: float = 0.01
    me: float = 1.0
    mi: float = 1.0
    sigma: float = 0.0
    ntimes: int = 4
    corr: float = 1.025
    periodic: tuple = (1, 1, 1)
    # deposit: 0 = FP32 atomics, 1 = int64 fixed point
    fixed: int = 0
    quirks: int = 0
    external_fields: int = 0
    ext: tuple = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    # particle capacity per species; 0 = 1.25 x the loaded count
    maxhlf: int = 0
    # GPU layout knobs (0 = automatic)
    sort_every: int = 1
    tile: tuple = (0, 0, 0)
    diag_every: int = 0
    # open-boundary window (x1in, x2in, y1in, y2in, z1in, z2in) when a
    # problem setup sets its own (None: the one allocate_particles derives)
    window: tuple | None = None

    # -- derived grid ----------------------------------------------------
    @property
    def nghost(self) -> int:
        return 5 if self.order == 1 else 7

    @property
    def nghostz(self) -> int:
        return 5 if self.dims == 2 else self.nghost

    @property
    def mx(self) -> int:
        return self.nx + self.nghost

    @property
    def my(self) -> int:
        return self.ny + self.nghost

    @property
    def mz(self) -> int:
        return 1 if self.dims == 2 else self.nz + self.nghostz

    @property
    def ncells(self) -> int:
        return self.mx * self.my * self.mz

    @property
    def interior_cells(self) -> int:
        return self.nx * self.ny * (self.nz if self.dims == 3 else 1)

    # -- derived particle constants (single precision, as the reference) --
    def _charges(self):
        c = f32(self.c)
        g0 = f32(self.gamma0)
        if g0 < 1:
            g0 = f32(np.sqrt(f32(1.0) / (f32(1.0) - g0 * g0)))
        omp = c / f32(self.c_omp)
        me, mi = f32(self.me), f32(self.mi)
        qe = -(omp * omp * g0) / ((f32(self.ppc0) * f32(0.5)) * (f32(1) + me / mi))
        qi = -qe
        me = me * abs(qi)
        mi = mi * abs(qi)
        return f32(qi), f32(qe), f32(qi / mi), f32(qe / me), g0

    @property
    def qi(self) -> float:
        return float(self._charges()[0])

    @property
    def qe(self) -> float:
        return float(self._charges()[1])

    @property
    def qmi(self) -> float:
        return float(self._charges()[2])

    @property
    def qme(self) -> float:
        return float(self._charges()[3])

    @property
    def gamma_drift(self) -> float:
        return float(self._charges()[4])

    @property
    def fx_shift(self) -> int:
        """Fixed-point scale 2^fx_shift: one unit is at most 2^-29 of the
        largest particle charge (finer than FP32 rounding of a deposit
        contribution), a single contribution stays below 2^30 units (so the
        device converts it with an exact 32-bit conversion), and a cell can
        sum ~2^33 full charges before the int64 accumulator overflows."""
        qmax = max(abs(self.qi), abs(self.qe))
        return 30 - int(math.ceil(math.log2(qmax)))

    def window_in(self):
        """x1in..z2in of allocate_particles (code/particles.F90:335-340);
        the reference's mx0 there already includes the ghosts."""
        if self.window is not None:
            return tuple(float(v) for v in self.window)
        ng, ngz = self.nghost, self.nghostz
        return (float(ng // 2 + 1), float(self.mx - ng // 2),
                float(ng // 2 + 1), float(self.my - ng // 2),
                float(ngz // 2 + 1), float((self.nz + ngz if self.dims == 3 else 1) - ngz // 2))

    # position window kept by the periodic wrap (deposit_particles,
    # code/particles_movedeposit.F90:1359-1374)
    @property
    def bounds(self):
        ng, ngz = self.nghost, self.nghostz
        minx, maxx = float(ng // 2 + 1), float(self.mx - ng // 2)
        miny, maxy = float(ng // 2 + 1), float(self.my - ng // 2)
        if self.dims == 3:
            minz, maxz = float(ngz // 2 + 1), float(self.mz - ngz // 2)
        else:
            minz, maxz = float(ngz // 2 + 1), float(ngz // 2 + 1) + 1.0
        return (minx, maxx), (miny, maxy), (minz, maxz)
