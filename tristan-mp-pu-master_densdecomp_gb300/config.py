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
    # deposit: 0 = tile sums rounded to FP32 (FP32 global atomics),
    # 1 = int64 fixed point (bit-reproducible)
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


def parse_input(path: str) -> dict:
    """The reference's `input` file as {section: {key: value}}: sections are
    `<name>` lines, entries `key = value`, `#` starts a comment (the format
    read by code/inputparser.c / code/inputparserf.F90); values parse as int
    or float where they can."""
    out: dict = {}
    sec = ""
    with open(path) as fh:
        for raw in fh:
            line = raw.split("#", 1)[0].strip()
            if not line:
                continue
            if line.startswith("<") and line.endswith(">"):
                sec = line[1:-1].strip()
                out.setdefault(sec, {})
                continue
            if "=" not in line:
                continue
            k, v = (t.strip() for t in line.split("=", 1))
            for conv in (int, float):
                try:
                    v = conv(v)
                    break
                except ValueError:
                    continue
            out.setdefault(sec, {})[k] = v
    return out


def from_input(path: str, dims: int, order: int, **overrides) -> SimConfig:
    """SimConfig from a reference `input` file. dims and order are the
    reference's compile-time choices (-DtwoD, -Ddd1/2/3); the keys used are
    those of read_input_grid, read_input_particles, read_input_algorithm and
    read_input_boundaries with the reference's defaults where absent
    (code/fields.F90:154-192, code/particles.F90:189-233,
    code/initialize.F90:293-305)."""
    d = parse_input(path)
    get = lambda sec, key, default: d.get(sec, {}).get(key, default)
    kw = dict(dims=dims, order=order,
              nx=int(get("grid", "mx0", 128)), ny=int(get("grid", "my0", 128)),
              nz=int(get("grid", "mz0", 1)) if dims == 3 else 1,
              c=float(get("time", "c", 0.45)),
              corr=float(get("algorithm", "Corr", 1.025)), ntimes=int(get("algorithm", "ntimes", 4)),
              ppc0=float(get("particles", "ppc0", 16)), gamma0=float(get("particles", "gamma0", 1.0)),
              delgam=float(get("particles", "delgam", 1e-4)), me=float(get("particles", "me", 1.0)),
              mi=float(get("particles", "mi", 1.0)), c_omp=float(get("particles", "c_omp", 10.0)),
              sigma=float(get("particles", "sigma", 0.0)),
              periodic=(int(get("boundaries", "periodicx", 1)), int(get("boundaries", "periodicy", 1)),
                        int(get("boundaries", "periodicz", 1))),
              external_fields=int(get("problem", "external_fields", 0)))
    kw.update(overrides)
    return SimConfig(**kw)
