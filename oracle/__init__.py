"""CPU oracle for the TRISTAN-MP hot path (test infrastructure only).

This package is the oracle used by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``. The GPU product path never imports
it. It wraps ``tristan_oracle.c`` (a restatement of the reference Fortran in
the reference's floating-point operation order) through ctypes.

Parity status: parity unpinned against reference outputs -- the reference
ships no tests or golden vectors and no Fortran compiler is available to run
it. The restatement is pinned by an independent pure-Python transliteration
(tests/golden/make_golden.py, bit-exact agreement) and by physics
known-answer tests.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "tristan_oracle.c")
LIB_SERIAL = os.path.join(BUILD, "libtristan_oracle.so")
LIB_OMP = os.path.join(BUILD, "libtristan_oracle_omp.so")

QUIRK_Q5_LHS = 1

PARTICLE_DTYPE = np.dtype(
    [("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("u", "<f4"), ("v", "<f4"), ("w", "<f4"),
     ("ch", "<f4"), ("ind", "<i4"), ("proc", "<i4"), ("splitlev", "<i4")]
)


def build(force: bool = False) -> None:
    """Compile the serial (parity) and OpenMP (CPU baseline) oracle libraries."""
    os.makedirs(BUILD, exist_ok=True)
    import platform
    stamp = os.path.join(BUILD, "host_arch")
    if not os.path.exists(stamp) or open(stamp).read().strip() != platform.machine():
        force = True
        with open(stamp, "w") as fh:
            fh.write(platform.machine() + "\n")
    common = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11",
              "-Wall", "-Wno-unused-variable", "-Wno-unused-but-set-variable", "-Wno-unknown-pragmas"]
    jobs = []
    for out, extra in ((LIB_SERIAL, []), (LIB_OMP, ["-fopenmp"])):
        if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(SRC):
            jobs.append(common + extra + [SRC, "-o", out, "-lm"])
    procs = [subprocess.Popen(j) for j in jobs]
    for p, j in zip(procs, jobs):
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: " + " ".join(j))


class to_particle(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("x", "y", "z", "u", "v", "w", "ch")] + \
               [(n, ctypes.c_int32) for n in ("ind", "proc", "splitlev")]


class to_state(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int32), ("order", ctypes.c_int32),
        ("mx", ctypes.c_int32), ("my", ctypes.c_int32), ("mz", ctypes.c_int32),
        ("nghost", ctypes.c_int32), ("nghostz", ctypes.c_int32),
        ("periodic", ctypes.c_int32 * 3),
        ("ntimes", ctypes.c_int32), ("quirks", ctypes.c_int32),
        ("c", ctypes.c_float), ("corr", ctypes.c_float), ("qi", ctypes.c_float),
        ("qe", ctypes.c_float), ("qmi", ctypes.c_float), ("qme", ctypes.c_float),
        ("external_fields", ctypes.c_int32), ("ext", ctypes.c_float * 6),
        ("x1in", ctypes.c_double), ("x2in", ctypes.c_double), ("y1in", ctypes.c_double),
        ("y2in", ctypes.c_double), ("z1in", ctypes.c_double), ("z2in", ctypes.c_double),
        ("mxcum", ctypes.c_int64), ("mycum", ctypes.c_int64), ("mzcum", ctypes.c_int64),
        ("fixed", ctypes.c_int32), ("fx_shift", ctypes.c_int32),
        ("maxhlf", ctypes.c_int64), ("ions", ctypes.c_int64), ("lecs", ctypes.c_int64),
        ("lap", ctypes.c_int64), ("lapreorder", ctypes.c_int64),
        ("p", ctypes.c_void_p), ("tempp", ctypes.c_void_p), ("pind", ctypes.c_void_p),
        ("pall", ctypes.c_void_p),
        ("ex", ctypes.c_void_p), ("ey", ctypes.c_void_p), ("ez", ctypes.c_void_p),
        ("bx", ctypes.c_void_p), ("by", ctypes.c_void_p), ("bz", ctypes.c_void_p),
        ("curx", ctypes.c_void_p), ("cury", ctypes.c_void_p), ("curz", ctypes.c_void_p),
        ("temp", ctypes.c_void_p),
        ("fx", ctypes.c_void_p), ("fy", ctypes.c_void_p), ("fz", ctypes.c_void_p),
        ("nionout", ctypes.c_int64), ("nlecout", ctypes.c_int64),
    ]


class to_diag(ctypes.Structure):
    _fields_ = [
        ("gauss_residual", ctypes.c_double), ("gauss_abs", ctypes.c_double),
        ("rho_norm", ctypes.c_double), ("e_field", ctypes.c_double), ("e_mag", ctypes.c_double),
        ("e_kin_ions", ctypes.c_double), ("e_kin_lecs", ctypes.c_double),
        ("p_part", ctypes.c_double * 3), ("p_field", ctypes.c_double * 3),
        ("charge_total", ctypes.c_double),
    ]


PDF_SZ = 1000


class to_shock(ctypes.Structure):
    _fields_ = [
        ("wall", ctypes.c_int32), ("walloc", ctypes.c_double),
        ("gammawall", ctypes.c_float), ("betawall", ctypes.c_float),
        ("cond_i1", ctypes.c_int32), ("cond_i2", ctypes.c_int32),
        ("edge_i1", ctypes.c_int32), ("edge_i2", ctypes.c_int32),
        ("edge", ctypes.c_float * 6),
        ("inject", ctypes.c_int32), ("xinject2", ctypes.c_double), ("betainj", ctypes.c_float),
        ("xinj_max", ctypes.c_double),
        ("ppc0", ctypes.c_float), ("gamma_drift", ctypes.c_float), ("weight", ctypes.c_float),
        ("y1", ctypes.c_float), ("y2", ctypes.c_float),
        ("pcosthmult", ctypes.c_float), ("sigma_nonzero", ctypes.c_int32),
        ("gamma_table_i", ctypes.c_float * PDF_SZ), ("pdf_table_i", ctypes.c_float * (PDF_SZ + 1)),
        ("gamma_table_e", ctypes.c_float * PDF_SZ), ("pdf_table_e", ctypes.c_float * (PDF_SZ + 1)),
        ("dseed", ctypes.c_double), ("totalpartnum", ctypes.c_int32), ("injected", ctypes.c_int64),
    ]


_libs: dict = {}
_lock = threading.Lock()


def load(openmp: bool = False) -> ctypes.CDLL:
    path = LIB_OMP if openmp else LIB_SERIAL
    with _lock:
        if path not in _libs:
            if not os.path.exists(path):
                build()
            lib = ctypes.CDLL(path)
            P = ctypes.POINTER(to_state)
            for name in ("to_move_particles", "to_deposit_particles", "to_fixed_to_float",
                         "to_reset_currents", "to_advance_b_halfstep", "to_advance_e_fullstep",
                         "to_add_current", "to_bc_b1", "to_bc_e1", "to_exchange_current",
                         "to_apply_filter1_opt", "to_reorder_particles", "to_reorder_particles_",
                         "to_step"):
                fn = getattr(lib, name)
                fn.argtypes = [P]
                fn.restype = None
            lib.to_mover.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_float]
            lib.to_mover.restype = None
            lib.to_densdecomp.argtypes = [P] + [ctypes.c_float] * 7
            lib.to_densdecomp.restype = None
            lib.to_diagnostics.argtypes = [P, ctypes.POINTER(to_diag)]
            lib.to_diagnostics.restype = None
            lib.to_charge_density.argtypes = [P, ctypes.c_void_p]
            lib.to_charge_density.restype = None
            lib.to_num_threads.argtypes = []
            lib.to_num_threads.restype = ctypes.c_int
            lib.to_meanq.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
            lib.to_meanq.restype = None
            lib.to_log10f.argtypes = [ctypes.c_float]
            lib.to_log10f.restype = ctypes.c_float
            lib.to_spectrum_dims.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int)]
            lib.to_spectrum_dims.restype = ctypes.c_int
            lib.to_spectrum_2d.argtypes = [P, ctypes.c_int] + [ctypes.c_void_p] * 5 + \
                [ctypes.POINTER(ctypes.c_float)] * 2
            lib.to_spectrum_2d.restype = None
            lib.to_output_dims.argtypes = [P, ctypes.c_int, ctypes.c_void_p]
            lib.to_output_dims.restype = ctypes.c_int
            lib.to_output_var.argtypes = [P] + [ctypes.c_int] * 5 + [ctypes.c_void_p]
            lib.to_output_var.restype = ctypes.c_int
            lib.to_output_particles.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                                                ctypes.c_void_p]
            lib.to_output_particles.restype = ctypes.c_int64
            lib.to_spectrum_x_bins.argtypes = [P]
            lib.to_spectrum_x_bins.restype = ctypes.c_int
            lib.to_spectrum_x.argtypes = [P, ctypes.c_int] + [ctypes.c_void_p] * 6 + \
                [ctypes.POINTER(ctypes.c_float)] * 2
            lib.to_spectrum_x.restype = None
            K = ctypes.POINTER(to_shock)
            lib.to_random.argtypes = [ctypes.POINTER(ctypes.c_double)]
            lib.to_random.restype = ctypes.c_float
            lib.to_poisson.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_double)]
            lib.to_poisson.restype = ctypes.c_float
            lib.to_sincosf.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
            lib.to_sincosf.restype = None
            lib.to_init_maxw_table.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_void_p,
                                               ctypes.c_void_p]
            lib.to_init_maxw_table.restype = None
            lib.to_maxwell_dist.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_double)] + \
                [ctypes.POINTER(ctypes.c_float)] * 3 + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_int]
            lib.to_maxwell_dist.restype = None
            lib.to_inject_plasma_region.argtypes = [P, K] + [ctypes.c_float] * 6
            lib.to_inject_plasma_region.restype = None
            lib.to_inject_plasma_region3.argtypes = [P, K] + [ctypes.c_float] * 8
            lib.to_inject_plasma_region3.restype = None
            for name in ("to_inject_particles_user", "to_particle_bc_user", "to_field_bc_user", "to_step_shock"):
                getattr(lib, name).argtypes = [P, K]
                getattr(lib, name).restype = None
            _libs[path] = lib
        return _libs[path]


FIELD_NAMES = ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz")


class OracleSim:
    """Owns the arrays of one oracle run (numpy), in the reference's layout.

    ``cfg`` is a ``tristan_gb300.SimConfig``-like object exposing dims,
    order, mx, my, mz (full extents), nghost, nghostz, periodic, ntimes, c,
    corr, qi, qe, qmi, qme, maxhlf, fixed, fx_shift, quirks, external_fields,
    ext.
    """

    def __init__(self, cfg, openmp: bool = False):
        self.cfg = cfg
        self.lib = load(openmp)
        n = cfg.mx * cfg.my * cfg.mz
        self.lot = n
        self.fields = {k: np.zeros(n, np.float32) for k in FIELD_NAMES}
        self.temp = np.zeros(n, np.float32)
        self.fixacc = [np.zeros(n, np.int64) for _ in range(3)]
        self.p = np.zeros(2 * cfg.maxhlf, PARTICLE_DTYPE)
        self.tempp = np.zeros(cfg.maxhlf, PARTICLE_DTYPE)
        self.pind = np.zeros(cfg.maxhlf, np.int32)
        self.pall = np.zeros(n + 1, np.int32)
        st = to_state()
        st.dims, st.order = cfg.dims, cfg.order
        st.mx, st.my, st.mz = cfg.mx, cfg.my, cfg.mz
        st.nghost, st.nghostz = cfg.nghost, cfg.nghostz
        for a in range(3):
            st.periodic[a] = int(cfg.periodic[a])
        st.ntimes, st.quirks = cfg.ntimes, cfg.quirks
        st.c, st.corr = cfg.c, cfg.corr
        st.qi, st.qe, st.qmi, st.qme = cfg.qi, cfg.qe, cfg.qmi, cfg.qme
        st.external_fields = int(cfg.external_fields)
        for a in range(6):
            st.ext[a] = float(cfg.ext[a])
        st.x1in, st.x2in, st.y1in, st.y2in, st.z1in, st.z2in = cfg.window_in()
        st.mxcum = st.mycum = st.mzcum = 0
        st.fixed, st.fx_shift = int(cfg.fixed), int(cfg.fx_shift)
        st.maxhlf = cfg.maxhlf
        st.ions = st.lecs = 0
        st.lap, st.lapreorder = 1, 0
        st.p = self.p.ctypes.data
        st.tempp = self.tempp.ctypes.data
        st.pind = self.pind.ctypes.data
        st.pall = self.pall.ctypes.data
        for k in FIELD_NAMES:
            setattr(st, k, self.fields[k].ctypes.data)
        st.temp = self.temp.ctypes.data
        st.fx, st.fy, st.fz = (a.ctypes.data for a in self.fixacc)
        self.st = st
        self.ptr = ctypes.pointer(st)

    # -- particles -----------------------------------------------------
    def set_particles(self, ions: np.ndarray, lecs: np.ndarray) -> None:
        mh = self.cfg.maxhlf
        assert len(ions) <= mh and len(lecs) <= mh
        self.p[: len(ions)] = ions
        self.p[mh: mh + len(lecs)] = lecs
        self.st.ions, self.st.lecs = len(ions), len(lecs)

    @property
    def ions(self) -> np.ndarray:
        return self.p[: self.st.ions]

    @property
    def lecs(self) -> np.ndarray:
        mh = self.cfg.maxhlf
        return self.p[mh: mh + self.st.lecs]

    def field(self, name: str) -> np.ndarray:
        c = self.cfg
        return self.fields[name].reshape(c.mz, c.my, c.mx)

    # -- phases ----------------------------------------------------------
    def call(self, name: str, *args):
        return getattr(self.lib, name)(self.ptr, *args)

    def step(self, n: int = 1) -> None:
        for _ in range(n):
            self.lib.to_step(self.ptr)

    def diagnostics(self) -> dict:
        d = to_diag()
        self.lib.to_diagnostics(self.ptr, ctypes.byref(d))
        out = {k: getattr(d, k) for k, _ in to_diag._fields_}
        out["p_part"] = list(d.p_part)
        out["p_field"] = list(d.p_field)
        return out

    # -- collisionless-shock hooks ------------------------------------------
    def shock_init(self, sh: dict) -> None:
        """to_shock from the dict of tristan_gb300.setups.shock_params; the
        Maxwell-Juttner tables are built by the restatement of
        init_maxw_table"""
        k = to_shock()
        for name, _ in to_shock._fields_:
            if name in sh and name != "edge":
                setattr(k, name, sh[name])
        for a in range(6):
            k.edge[a] = float(sh["edge"][a])
        self.lib.to_init_maxw_table(float(sh["delgam_i"]), int(self.cfg.dims), float(sh["pcosthmult"]),
                                    ctypes.addressof(k.gamma_table_i), ctypes.addressof(k.pdf_table_i))
        self.lib.to_init_maxw_table(float(sh["delgam_e"]), int(self.cfg.dims), float(sh["pcosthmult"]),
                                    ctypes.addressof(k.gamma_table_e), ctypes.addressof(k.pdf_table_e))
        self.shock = k
        self.kptr = ctypes.pointer(k)

    def inject_region(self, x1, x2, y1, y2, ppc, weight=1.0) -> None:
        self.lib.to_inject_plasma_region(self.ptr, self.kptr, x1, x2, y1, y2, ppc, weight)

    def inject_region3(self, x1, x2, y1, y2, z1, z2, ppc, weight=1.0) -> None:
        self.lib.to_inject_plasma_region3(self.ptr, self.kptr, x1, x2, y1, y2, z1, z2, ppc, weight)

    def step_shock(self, n: int = 1) -> None:
        for _ in range(n):
            self.lib.to_step_shock(self.ptr, self.kptr)

    def shock_call(self, name: str) -> None:
        getattr(self.lib, name)(self.ptr, self.kptr)

    def meanq(self, kind: int, idx: int = 2, idy: int = 2, idz: int = 2):
        num = np.zeros(self.lot, np.float32)
        den = np.zeros(self.lot, np.float32)
        self.lib.to_meanq(self.ptr, kind, idx, idy, idz if self.cfg.dims == 3 else 0, num.ctypes.data,
                          den.ctypes.data)
        return num, den

    def spectrum(self, gambins: int = 200) -> dict:
        nx, ny = ctypes.c_int(), ctypes.c_int()
        self.lib.to_spectrum_dims(self.ptr, gambins, ctypes.byref(nx), ctypes.byref(ny))
        si = np.zeros((gambins, ny.value, nx.value), np.float32)
        se = np.zeros_like(si)
        xg = np.zeros(gambins, np.float32)
        xs = np.zeros(nx.value, np.float32)
        ys = np.zeros(ny.value, np.float32)
        gmin, gmax = ctypes.c_float(), ctypes.c_float()
        self.lib.to_spectrum_2d(self.ptr, gambins, si.ctypes.data, se.ctypes.data, xg.ctypes.data, xs.ctypes.data,
                                ys.ctypes.data, ctypes.byref(gmin), ctypes.byref(gmax))
        return dict(ions=si, lecs=se, xgamma=xg, xslice=xs, yslice=ys, gammin=gmin.value, gammax=gmax.value)

    def output_var(self, var: int, istep: int, idx: int = 2, idy: int = 2, idz: int = 2) -> np.ndarray:
        """output_tot: one variable sampled every istep nodes, (nz, ny, nx)"""
        dims = np.zeros(3, np.int32)
        self.lib.to_output_dims(self.ptr, istep, dims.ctypes.data)
        out = np.zeros(int(dims.prod()), np.float32)
        self.lib.to_output_var(self.ptr, var, istep, idx, idy, idz if self.cfg.dims == 3 else 0, out.ctypes.data)
        return out.reshape(dims[2], dims[1], dims[0])

    def output_particles(self, species: int, stride: int) -> dict:
        """output_tot's particle sample: x, y, z, u, v, w, ch, gamma, ind, proc"""
        total = self.lib.to_output_particles(self.ptr, species, stride, 0, None, None)
        vals = np.zeros((8, max(total, 1)), np.float32)
        ids = np.zeros((2, max(total, 1)), np.int32)
        self.lib.to_output_particles(self.ptr, species, stride, max(total, 1), vals.ctypes.data, ids.ctypes.data)
        names = ("x", "y", "z", "u", "v", "w", "ch", "gamma")
        out = {k: vals[i, :total] for i, k in enumerate(names)}
        out["ind"], out["proc"] = ids[0, :total], ids[1, :total]
        return out

    def spectrum_x(self, gambins: int = 200) -> dict:
        """save_spectrum: per x slice, lab-frame and flow-frame spectra"""
        nb = self.lib.to_spectrum_x_bins(self.ptr)
        out = {k: np.zeros((gambins, nb), np.float32) for k in ("ions", "lecs", "ions_rest", "lecs_rest")}
        xg = np.zeros(gambins, np.float32)
        xs = np.zeros(nb, np.float32)
        gmin, gmax = ctypes.c_float(), ctypes.c_float()
        self.lib.to_spectrum_x(self.ptr, gambins, out["ions"].ctypes.data, out["lecs"].ctypes.data,
                               out["ions_rest"].ctypes.data, out["lecs_rest"].ctypes.data, xg.ctypes.data,
                               xs.ctypes.data, ctypes.byref(gmin), ctypes.byref(gmax))
        return dict(out, xgamma=xg, xslice=xs, gammin=gmin.value, gammax=gmax.value)

    def charge_density(self) -> np.ndarray:
        rho = np.zeros(self.lot, np.float64)
        self.lib.to_charge_density(self.ptr, rho.ctypes.data)
        return rho
