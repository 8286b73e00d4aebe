"""Host-side mirror of the reference's per-step subroutines over the C-ABI.

``GpuSim`` owns the host arrays the reference keeps in its modules (fields
``ex..curz`` in Fortran order, the particle array ``p`` with ions at
``p[0:ions]`` and electrons at ``p[maxhlf:maxhlf+lecs]``) and calls
``libtristan_gpu.so`` (declared in include/tristan_gpu.h) through ctypes. Its
method names follow the reference subroutines: ``bc_b1``, ``bc_e1``,
``advance_Bhalfstep``, ``advance_Efield``, ``move_particles``,
``reset_currents``, ``deposit_particles``, ``exchange_current``,
``apply_filter1_opt``, ``add_current``, ``reorder_particles`` and ``step``
(one lap of the main loop). Errors raise ``TristanGpuError`` with the
library's message, as the reference prints and stops.

There is no CPU fallback: if the library is not built or no GPU is present
the constructor raises.
"""
from __future__ import annotations

import ctypes
import mmap
import os

import numpy as np

from .config import SimConfig
from .setups import PARTICLE_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libtristan_gpu.so")

TG_OK, TG_ERR_ARG, TG_ERR_CUDA, TG_ERR_OVERFLOW, TG_ERR_BOUNDS, TG_ERR_NAN, TG_ERR_STATE = range(7)
SYNC_E, SYNC_B, SYNC_CUR, SYNC_PARTICLES, SYNC_ALL = 1, 2, 4, 8, 15
QUIRK_Q5_LHS = 1
DEPOSIT_FP32, DEPOSIT_FIXED = 0, 1

FIELD_NAMES = ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz")


class TristanGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[tg error {code}] {msg}")
        self.code = code


class tg_config(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int32), ("order", ctypes.c_int32),
        ("mx", ctypes.c_int32), ("my", ctypes.c_int32), ("mz", ctypes.c_int32),
        ("nghost", ctypes.c_int32), ("nghostz", ctypes.c_int32),
        ("periodic", ctypes.c_int32 * 3), ("ntimes", ctypes.c_int32), ("quirks", ctypes.c_int32),
        ("c", ctypes.c_float), ("corr", ctypes.c_float), ("qi", ctypes.c_float), ("qe", ctypes.c_float),
        ("qmi", ctypes.c_float), ("qme", ctypes.c_float),
        ("external_fields", ctypes.c_int32), ("ext", ctypes.c_float * 6),
        ("x1in", ctypes.c_double), ("x2in", ctypes.c_double), ("y1in", ctypes.c_double),
        ("y2in", ctypes.c_double), ("z1in", ctypes.c_double), ("z2in", ctypes.c_double),
        ("mxcum", ctypes.c_int64), ("mycum", ctypes.c_int64), ("mzcum", ctypes.c_int64),
        ("deposit_mode", ctypes.c_int32), ("fx_shift", ctypes.c_int32),
        ("maxhlf", ctypes.c_int64),
        ("sort_every", ctypes.c_int32), ("tile", ctypes.c_int32 * 3), ("device", ctypes.c_int32),
        ("diag_every", ctypes.c_int32),
    ]


class tg_shock(ctypes.Structure):
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
        ("delgam_i", ctypes.c_float), ("delgam_e", ctypes.c_float),
        ("pcosthmult", ctypes.c_float), ("sigma_nonzero", ctypes.c_int32),
        ("dseed", ctypes.c_double), ("totalpartnum", ctypes.c_int32),
    ]


def make_tg_shock(sh: dict) -> tg_shock:
    """tg_shock from the dict of setups.shock_params"""
    k = tg_shock()
    for name, _ in tg_shock._fields_:
        if name == "edge":
            for a in range(6):
                k.edge[a] = float(sh["edge"][a])
        else:
            setattr(k, name, sh[name])
    return k


class tg_restart_meta(ctypes.Structure):
    _fields_ = [
        ("dseed", ctypes.c_double), ("lap", ctypes.c_int32),
        ("xinject", ctypes.c_double), ("xinject2", ctypes.c_double), ("xinject3", ctypes.c_double),
        ("leftwall", ctypes.c_float), ("walloc", ctypes.c_double),
        ("totalpartnum", ctypes.c_int32), ("maxptl", ctypes.c_int32), ("max_subrecord", ctypes.c_int64),
    ]


class tg_diag(ctypes.Structure):
    _fields_ = [
        ("gauss_residual", ctypes.c_double), ("gauss_abs", ctypes.c_double),
        ("rho_norm", ctypes.c_double), ("e_field", ctypes.c_double), ("e_mag", ctypes.c_double),
        ("e_kin_ions", ctypes.c_double), ("e_kin_lecs", ctypes.c_double),
        ("p_part", ctypes.c_double * 3), ("p_field", ctypes.c_double * 3),
        ("charge_total", ctypes.c_double),
    ]


_lib = None

ENTRY_POINTS = (
    "tg_init", "tg_finalize", "tg_last_error", "tg_bind_fields", "tg_bind_particles",
    "tg_sync_from_host", "tg_sync_to_host", "tg_bc_b1", "tg_bc_e1", "tg_advance_b_half",
    "tg_advance_e", "tg_move", "tg_reset_currents", "tg_deposit", "tg_fold_currents",
    "tg_filter", "tg_add_current", "tg_reorder", "tg_step", "tg_step_host", "tg_pin_host", "tg_set_host_parts", "tg_diag_fp64", "tg_synchronize",
    "tg_get_counts", "tg_device_fields", "tg_stream", "tg_kernels_per_step", "tg_diag_history",
    "tg_enable_timing", "tg_phase_times", "tg_step_timed", "tg_filter_noalloc", "tg_autotune",
    "tg_ens_init", "tg_ens_finalize", "tg_ens_last_error", "tg_ens_bind_fields", "tg_ens_bind_particles",
    "tg_ens_sync_from_host", "tg_ens_sync_to_host", "tg_ens_step", "tg_ens_step_timed", "tg_ens_diag_fp64",
    "tg_ens_get_counts", "tg_ens_synchronize", "tg_ens_kernels_per_step", "tg_ens_autotune",
    "tg_shock_init", "tg_shock_get", "tg_inject_region", "tg_particle_bc", "tg_field_bc", "tg_inject",
    "tg_write_restart", "tg_read_restart", "tg_moments", "tg_spectrum_dims", "tg_spectrum", "tg_spectrum_x_bins",
    "tg_spectrum_x", "tg_output_dims", "tg_output_var", "tg_output_particles",
)
# grid moments of meanq_fld_cur (code/output.F90:5222-5482), by the reference's names
MOMENTS = ("tdens", "idens", "tbetx", "tbety", "tbetz", "ibetx", "ibety", "ibetz", "tmomx", "tmomy", "tmomz",
           "imomx", "imomy", "imomz", "eener", "iener")
# tg_phase_times' phases, grouped as the reference's per-lap timers
# (code/communications.F90:242-326): Field slv = fields_pre + fields_post +
# add_current, Mover + Deposit = particles, Currnt exch = fold, Filter =
# filter, Reorder = sort; diag has no counterpart
PHASES = ("fields_pre", "particles", "fields_post", "fold", "filter", "add_current", "sort", "diag")


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libtristan_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    lib.tg_init.argtypes = [ctypes.POINTER(tg_config), ctypes.POINTER(P)]
    lib.tg_init.restype = ctypes.c_int
    lib.tg_finalize.argtypes = [P]
    lib.tg_finalize.restype = None
    lib.tg_last_error.argtypes = [P]
    lib.tg_last_error.restype = ctypes.c_char_p
    lib.tg_bind_fields.argtypes = [P] + [P] * 9
    lib.tg_bind_fields.restype = ctypes.c_int
    lib.tg_bind_particles.argtypes = [P, P, P, P]
    lib.tg_bind_particles.restype = ctypes.c_int
    for n in ("tg_sync_from_host", "tg_sync_to_host"):
        getattr(lib, n).argtypes = [P, ctypes.c_uint]
        getattr(lib, n).restype = ctypes.c_int
    for n in ("tg_bc_b1", "tg_bc_e1", "tg_advance_b_half", "tg_advance_e", "tg_move", "tg_reset_currents",
              "tg_deposit", "tg_fold_currents", "tg_filter", "tg_add_current", "tg_synchronize"):
        getattr(lib, n).argtypes = [P]
        getattr(lib, n).restype = ctypes.c_int
    lib.tg_reorder.argtypes = [P, ctypes.c_int32, ctypes.c_int32]
    lib.tg_reorder.restype = ctypes.c_int
    lib.tg_step.argtypes = [P, ctypes.c_int32]
    lib.tg_step.restype = ctypes.c_int
    lib.tg_step_host.argtypes = [P, ctypes.c_int32]
    lib.tg_step_host.restype = ctypes.c_int
    lib.tg_pin_host.argtypes = [P]
    lib.tg_pin_host.restype = ctypes.c_int
    lib.tg_set_host_parts.argtypes = [P, ctypes.c_int32]
    lib.tg_set_host_parts.restype = ctypes.c_int
    lib.tg_diag_fp64.argtypes = [P, ctypes.POINTER(tg_diag)]
    lib.tg_diag_fp64.restype = ctypes.c_int
    lib.tg_get_counts.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    lib.tg_get_counts.restype = ctypes.c_int
    lib.tg_device_fields.argtypes = [P, ctypes.POINTER(P)]
    lib.tg_device_fields.restype = ctypes.c_int
    lib.tg_stream.argtypes = [P]
    lib.tg_stream.restype = P
    lib.tg_kernels_per_step.argtypes = [P]
    lib.tg_kernels_per_step.restype = ctypes.c_int32
    lib.tg_diag_history.argtypes = [P, ctypes.c_void_p, ctypes.c_int32]
    lib.tg_diag_history.restype = ctypes.c_int
    lib.tg_step_timed.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)]
    lib.tg_step_timed.restype = ctypes.c_int
    lib.tg_autotune.argtypes = [ctypes.POINTER(tg_config), P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_float), P, ctypes.c_int32]
    lib.tg_autotune.restype = ctypes.c_int
    lib.tg_enable_timing.argtypes = [P, ctypes.c_int32]
    lib.tg_enable_timing.restype = ctypes.c_int
    lib.tg_phase_times.argtypes = [P, ctypes.c_void_p, ctypes.c_int32]
    lib.tg_phase_times.restype = ctypes.c_int
    # collisionless-shock hooks
    lib.tg_shock_init.argtypes = [P, ctypes.POINTER(tg_shock)]
    lib.tg_shock_init.restype = ctypes.c_int
    lib.tg_shock_get.argtypes = [P, ctypes.POINTER(tg_shock)]
    lib.tg_shock_get.restype = ctypes.c_int
    lib.tg_inject_region.argtypes = [P] + [ctypes.c_float] * 6
    lib.tg_inject_region.restype = ctypes.c_int
    for n in ("tg_particle_bc", "tg_field_bc", "tg_inject"):
        getattr(lib, n).argtypes = [P]
        getattr(lib, n).restype = ctypes.c_int
    lib.tg_spectrum_dims.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    lib.tg_spectrum_dims.restype = ctypes.c_int
    lib.tg_spectrum.argtypes = [P, ctypes.c_int32] + [P] * 6
    lib.tg_spectrum.restype = ctypes.c_int
    lib.tg_output_dims.argtypes = [P, ctypes.c_int32, P]
    lib.tg_output_dims.restype = ctypes.c_int
    lib.tg_output_var.argtypes = [P] + [ctypes.c_int32] * 5 + [P]
    lib.tg_output_var.restype = ctypes.c_int
    lib.tg_output_particles.argtypes = [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, P, P,
                                        ctypes.POINTER(ctypes.c_int64)]
    lib.tg_output_particles.restype = ctypes.c_int
    lib.tg_spectrum_x_bins.argtypes = [P, ctypes.POINTER(ctypes.c_int32)]
    lib.tg_spectrum_x_bins.restype = ctypes.c_int
    lib.tg_spectrum_x.argtypes = [P, ctypes.c_int32] + [P] * 7
    lib.tg_spectrum_x.restype = ctypes.c_int
    lib.tg_moments.argtypes = [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, P, P]
    lib.tg_moments.restype = ctypes.c_int
    lib.tg_write_restart.argtypes = [P, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(tg_restart_meta)]
    lib.tg_write_restart.restype = ctypes.c_int
    lib.tg_read_restart.argtypes = [P, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(tg_restart_meta)]
    lib.tg_read_restart.restype = ctypes.c_int
    # batched ensemble
    lib.tg_ens_init.argtypes = [ctypes.POINTER(tg_config), ctypes.c_int32, ctypes.POINTER(P)]
    lib.tg_ens_init.restype = ctypes.c_int
    lib.tg_ens_finalize.argtypes = [P]
    lib.tg_ens_finalize.restype = None
    lib.tg_ens_last_error.argtypes = [P]
    lib.tg_ens_last_error.restype = ctypes.c_char_p
    lib.tg_ens_bind_fields.argtypes = [P, ctypes.c_int32] + [P] * 9
    lib.tg_ens_bind_fields.restype = ctypes.c_int
    lib.tg_ens_bind_particles.argtypes = [P, ctypes.c_int32, P, P, P]
    lib.tg_ens_bind_particles.restype = ctypes.c_int
    for n in ("tg_ens_sync_from_host", "tg_ens_sync_to_host"):
        getattr(lib, n).argtypes = [P, ctypes.c_uint]
        getattr(lib, n).restype = ctypes.c_int
    lib.tg_ens_step.argtypes = [P, ctypes.c_int32]
    lib.tg_ens_step.restype = ctypes.c_int
    lib.tg_ens_step_timed.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)]
    lib.tg_ens_step_timed.restype = ctypes.c_int
    lib.tg_ens_diag_fp64.argtypes = [P, ctypes.c_int32, ctypes.POINTER(tg_diag)]
    lib.tg_ens_diag_fp64.restype = ctypes.c_int
    lib.tg_ens_get_counts.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64)]
    lib.tg_ens_get_counts.restype = ctypes.c_int
    lib.tg_ens_synchronize.argtypes = [P]
    lib.tg_ens_synchronize.restype = ctypes.c_int
    lib.tg_ens_kernels_per_step.argtypes = [P]
    lib.tg_ens_kernels_per_step.restype = ctypes.c_int32
    lib.tg_ens_autotune.argtypes = [ctypes.POINTER(tg_config), ctypes.c_int32, P, P, P, ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_float), P, ctypes.c_int32]
    lib.tg_ens_autotune.restype = ctypes.c_int
    _lib = lib
    return lib


def make_tg_config(cfg: SimConfig, device: int = 0) -> tg_config:
    c = tg_config()
    c.dims, c.order = cfg.dims, cfg.order
    c.mx, c.my, c.mz = cfg.mx, cfg.my, cfg.mz
    c.nghost, c.nghostz = cfg.nghost, cfg.nghostz
    for a in range(3):
        c.periodic[a] = int(cfg.periodic[a])
    c.ntimes, c.quirks = cfg.ntimes, cfg.quirks
    c.c, c.corr = cfg.c, cfg.corr
    c.qi, c.qe, c.qmi, c.qme = cfg.qi, cfg.qe, cfg.qmi, cfg.qme
    c.external_fields = int(cfg.external_fields)
    for a in range(6):
        c.ext[a] = float(cfg.ext[a])
    c.x1in, c.x2in, c.y1in, c.y2in, c.z1in, c.z2in = cfg.window_in()
    c.mxcum = c.mycum = c.mzcum = 0
    c.deposit_mode = DEPOSIT_FIXED if cfg.fixed else DEPOSIT_FP32
    c.fx_shift = cfg.fx_shift
    c.maxhlf = cfg.maxhlf
    c.sort_every = max(1, int(cfg.sort_every))
    for a in range(3):
        c.tile[a] = int(cfg.tile[a])
    c.device = device
    c.diag_every = int(cfg.diag_every)
    return c


def autotune(cfg: SimConfig, ions: np.ndarray, lecs: np.ndarray, laps: int = 2, device: int = 0):
    """Pick tile shape and re-sort cadence for this domain and plasma
    (tg_autotune); updates cfg.tile / cfg.sort_every in place and returns
    (best ms per lap, table of (tx, ty, tz, sort_every, ms))."""
    lib = load_library()
    if cfg.maxhlf == 0:
        cfg.maxhlf = int(max(len(ions), len(lecs)) * 1.25) + 1024
    p = np.zeros(2 * cfg.maxhlf, PARTICLE_DTYPE)
    p[: len(ions)] = ions
    p[cfg.maxhlf: cfg.maxhlf + len(lecs)] = lecs
    c = make_tg_config(cfg, device)
    best = ctypes.c_float()
    table = np.zeros((64, 5), np.float32)
    rows = lib.tg_autotune(ctypes.byref(c), p.ctypes.data, len(ions), len(lecs), int(laps), ctypes.byref(best),
                           table.ctypes.data, 64)
    if rows < 0:
        raise TristanGpuError(-rows, "autotune: no candidate ran")
    cfg.tile = (int(c.tile[0]), int(c.tile[1]), int(c.tile[2]))
    cfg.sort_every = int(c.sort_every)
    return float(best.value), table[:rows]


_cudart = None


def _cudart_lib():
    global _cudart
    if _cudart is None:
        load_library()  # pulls libcudart in with the C-ABI library
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                _cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if _cudart is None:
            raise RuntimeError("libcudart not found")
        _cudart.cudaHostRegister.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint]
        _cudart.cudaHostRegister.restype = ctypes.c_int
        _cudart.cudaHostUnregister.argtypes = [ctypes.c_void_p]
        _cudart.cudaHostUnregister.restype = ctypes.c_int
    return _cudart


def _huge_page_bytes() -> int:
    try:
        with open("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size") as f:
            return max(int(f.read()), 2 << 20)
    except (OSError, ValueError):
        return 2 << 20


def _host_array(n: int, dtype, pinned: bool) -> np.ndarray:
    """zeroed host array of n elements; when it is to be page-locked, on
    anonymous memory advised for transparent huge pages and aligned to them
    (page-locked base pages sustain fewer bytes per second over the host
    link when both directions run at once)"""
    dtype = np.dtype(dtype)
    if not pinned or n == 0:
        return np.zeros(n, dtype)
    nbytes = n * dtype.itemsize
    huge = _huge_page_bytes()
    m = mmap.mmap(-1, nbytes + huge)  # anonymous, zero-filled; address space only until touched
    if hasattr(mmap, "MADV_HUGEPAGE"):
        m.madvise(mmap.MADV_HUGEPAGE)
    raw = np.frombuffer(m, np.uint8)  # keeps the mapping alive
    off = (-raw.ctypes.data) % huge
    return raw[off: off + nbytes].view(dtype)


def huge_page_fraction(arrays) -> float | None:
    """share of the memory mappings holding `arrays` that the kernel backs
    with transparent huge pages (AnonHugePages / Size in /proc/self/smaps);
    None where smaps cannot be read"""
    spans = [(a.ctypes.data, a.ctypes.data + a.nbytes) for a in arrays if a.nbytes]
    if not spans:
        return None
    try:
        with open("/proc/self/smaps") as f:
            lines = f.read().splitlines()
    except OSError:
        return None
    size = huge = 0
    hit = False
    for line in lines:
        head = line.split(None, 1)[0] if line else ""
        if "-" in head and ":" not in head:
            try:
                lo, hi = (int(v, 16) for v in head.split("-"))
            except ValueError:
                hit = False
                continue
            hit = any(lo < e and s < hi for s, e in spans)
        elif hit and head == "Size:":
            size += int(line.split()[1])
        elif hit and head == "AnonHugePages:":
            huge += int(line.split()[1])
    return huge / size if size else None


class GpuSim:
    """One device domain plus the host arrays it syncs with. ``pinned``
    puts the host arrays on huge pages and page-locks them
    (cudaHostRegister) for full-speed copies."""

    def __init__(self, cfg: SimConfig, device: int = 0, pinned: bool = False):
        self.cfg = cfg
        self.lib = load_library()
        self.tcfg = make_tg_config(cfg, device)
        h = ctypes.c_void_p()
        rc = self.lib.tg_init(ctypes.byref(self.tcfg), ctypes.byref(h))
        if rc != TG_OK:
            raise TristanGpuError(rc, self.lib.tg_last_error(None).decode())
        self.h = h
        n = cfg.mx * cfg.my * cfg.mz
        self.lot = n
        self.fields = {k: _host_array(n, np.float32, pinned) for k in FIELD_NAMES}
        self.p = _host_array(2 * cfg.maxhlf, PARTICLE_DTYPE, pinned)
        self._ions = ctypes.c_int32(0)
        self._lecs = ctypes.c_int32(0)
        self._pinned = []
        if pinned:
            rt = _cudart_lib()
            for arr in [self.p] + [self.fields[k] for k in FIELD_NAMES]:
                if rt.cudaHostRegister(arr.ctypes.data, arr.nbytes, 0) != 0:
                    raise TristanGpuError(TG_ERR_CUDA, "cudaHostRegister failed")
                self._pinned.append(arr)
        self._check(self.lib.tg_bind_fields(self.h, *[self.fields[k].ctypes.data for k in FIELD_NAMES]))
        self._check(self.lib.tg_bind_particles(self.h, self.p.ctypes.data, ctypes.addressof(self._ions),
                                               ctypes.addressof(self._lecs)))

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.tg_finalize(self.h)
            self.h = None
            for arr in getattr(self, "_pinned", []):
                _cudart_lib().cudaHostUnregister(arr.ctypes.data)
            self._pinned = []

    def host_huge_fraction(self) -> float | None:
        """share of the host arrays' mappings on transparent huge pages"""
        return huge_page_fraction([self.p] + [self.fields[k] for k in FIELD_NAMES])

    def host_bytes(self, mask: int) -> int:
        """bytes one sync of `mask` moves (particles at the current counts)"""
        n = 0
        per = self.lot * 4
        if mask & SYNC_E:
            n += 3 * per
        if mask & SYNC_B:
            n += 3 * per
        if mask & SYNC_CUR:
            n += 3 * per
        if mask & SYNC_PARTICLES:
            n += (self._ions.value + self._lecs.value) * PARTICLE_DTYPE.itemsize
        return n

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != TG_OK:
            raise TristanGpuError(rc, self.lib.tg_last_error(self.h).decode())

    # -- host <-> device -----------------------------------------------------
    def set_particles(self, ions: np.ndarray, lecs: np.ndarray, upload: bool = True) -> None:
        mh = self.cfg.maxhlf
        if len(ions) > mh or len(lecs) > mh:
            raise TristanGpuError(TG_ERR_OVERFLOW, "particle count exceeds maxhlf")
        self.p[: len(ions)] = ions
        self.p[mh: mh + len(lecs)] = lecs
        self._ions.value, self._lecs.value = len(ions), len(lecs)
        if upload:
            self.sync_from_host(SYNC_PARTICLES)

    def set_fields(self, **arrays) -> None:
        for k, v in arrays.items():
            self.fields[k][:] = np.asarray(v, np.float32).ravel()

    def sync_from_host(self, mask: int = SYNC_ALL) -> None:
        self._check(self.lib.tg_sync_from_host(self.h, mask))

    def sync_to_host(self, mask: int = SYNC_ALL) -> None:
        self._check(self.lib.tg_sync_to_host(self.h, mask))

    @property
    def ions(self) -> np.ndarray:
        return self.p[: self._ions.value]

    @property
    def lecs(self) -> np.ndarray:
        mh = self.cfg.maxhlf
        return self.p[mh: mh + self._lecs.value]

    def counts(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.tg_get_counts(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # -- the reference's per-lap subroutines ------------------------------
    def bc_b1(self):
        self._check(self.lib.tg_bc_b1(self.h))

    def bc_e1(self):
        self._check(self.lib.tg_bc_e1(self.h))

    def advance_Bhalfstep(self):
        self._check(self.lib.tg_advance_b_half(self.h))

    def advance_Efield(self):
        self._check(self.lib.tg_advance_e(self.h))

    def move_particles(self):
        self._check(self.lib.tg_move(self.h))

    def reset_currents(self):
        self._check(self.lib.tg_reset_currents(self.h))

    def deposit_particles(self):
        self._check(self.lib.tg_deposit(self.h))

    def exchange_current(self):
        self._check(self.lib.tg_fold_currents(self.h))

    def apply_filter1_opt(self):
        self._check(self.lib.tg_filter(self.h))

    def add_current(self):
        self._check(self.lib.tg_add_current(self.h))

    def reorder_particles(self, lap: int, force: bool = False):
        self._check(self.lib.tg_reorder(self.h, int(lap), 1 if force else 0))

    def step(self, n: int = 1):
        self._check(self.lib.tg_step(self.h, int(n)))

    def step_host(self, n: int = 1):
        """n main-loop passes with the host arrays as the state (tg_step_host):
        E, B and the records up, the lap, everything back, every lap"""
        self._check(self.lib.tg_step_host(self.h, int(n)))

    def pin_host(self):
        """page-lock the bound host arrays from the library (tg_pin_host)"""
        self._check(self.lib.tg_pin_host(self.h))

    def set_host_parts(self, parts: int):
        """parts per species for the overlapped step_host (tg_set_host_parts;
        0: by size)"""
        self._check(self.lib.tg_set_host_parts(self.h, int(parts)))

    def step_timed(self, n: int) -> float:
        """n laps bracketed by CUDA events on the library's stream; ms"""
        ms = ctypes.c_float()
        self._check(self.lib.tg_step_timed(self.h, int(n), ctypes.byref(ms)))
        return float(ms.value)

    def synchronize(self):
        self._check(self.lib.tg_synchronize(self.h))

    def kernels_per_step(self) -> int:
        return int(self.lib.tg_kernels_per_step(self.h))

    def diagnostics(self) -> dict:
        d = tg_diag()
        self._check(self.lib.tg_diag_fp64(self.h, ctypes.byref(d)))
        return _diag_dict(d)

    DIAG_KEYS = ("res2", "rho2", "charge_total", "e_field", "e_mag", "e_kin_ions", "e_kin_lecs",
                 "px", "py", "pz", "fx", "fy", "fz")

    def diag_history(self, n: int) -> np.ndarray:
        out = np.zeros((n, 16), np.float64)
        got = self.lib.tg_diag_history(self.h, out.ctypes.data, int(n))
        if got < 0:
            self._check(got)
        return out[:got]

    def enable_timing(self, on: bool = True):
        self._check(self.lib.tg_enable_timing(self.h, 1 if on else 0))

    def phase_times(self) -> dict:
        ms = np.zeros(len(PHASES), np.float32)
        self._check(self.lib.tg_phase_times(self.h, ms.ctypes.data, len(PHASES)))
        return {k: float(v) for k, v in zip(PHASES, ms)}

    def field(self, name: str) -> np.ndarray:
        c = self.cfg
        return self.fields[name].reshape(c.mz, c.my, c.mx)

    # -- collisionless-shock hooks -------------------------------------------
    def shock_init(self, sh: dict):
        self._shock = make_tg_shock(sh)
        self._check(self.lib.tg_shock_init(self.h, ctypes.byref(self._shock)))

    def shock_state(self) -> dict:
        k = tg_shock()
        self._check(self.lib.tg_shock_get(self.h, ctypes.byref(k)))
        return {n: (list(k.edge) if n == "edge" else getattr(k, n)) for n, _ in tg_shock._fields_}

    def inject_region(self, x1, x2, y1, y2, ppc, weight=1.0):
        self._check(self.lib.tg_inject_region(self.h, x1, x2, y1, y2, ppc, weight))

    def particle_bc_user(self):
        self._check(self.lib.tg_particle_bc(self.h))

    def field_bc_user(self):
        self._check(self.lib.tg_field_bc(self.h))

    def inject_particles_user(self):
        self._check(self.lib.tg_inject(self.h))

    # -- output moments (meanq_fld_cur) ----------------------------------------
    def meanq(self, name: str, idx: int = 2, idy: int = 2, idz: int = 2):
        """(moment, box-averaged weight), each mx*my*mz floats"""
        num = np.zeros(self.lot, np.float32)
        den = np.zeros(self.lot, np.float32)
        self._check(self.lib.tg_moments(self.h, MOMENTS.index(name), idx, idy, idz, num.ctypes.data,
                                        den.ctypes.data))
        return num, den

    def spectrum(self, gambins: int = 200) -> dict:
        """flow-frame energy spectra per slice (save_spectrum_2d)"""
        nx, ny = ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.tg_spectrum_dims(self.h, gambins, ctypes.byref(nx), ctypes.byref(ny)))
        si = np.zeros((gambins, ny.value, nx.value), np.float32)
        se = np.zeros_like(si)
        xg = np.zeros(gambins, np.float32)
        xs = np.zeros(nx.value, np.float32)
        ys = np.zeros(ny.value, np.float32)
        gr = np.zeros(2, np.float32)
        self._check(self.lib.tg_spectrum(self.h, gambins, si.ctypes.data, se.ctypes.data, xg.ctypes.data,
                                         xs.ctypes.data, ys.ctypes.data, gr.ctypes.data))
        return dict(ions=si, lecs=se, xgamma=xg, xslice=xs, yslice=ys, gammin=float(gr[0]), gammax=float(gr[1]))

    # .tot. output variables (output_tot): E, B, currents, moments by name
    OUTPUT_VARS = {"ex": 0, "ey": 1, "ez": 2, "bx": 3, "by": 4, "bz": 5, "jx": 6, "jy": 7, "jz": 8}

    def output_var(self, var, istep: int, idx: int = 2, idy: int = 2, idz: int = 2) -> np.ndarray:
        """one .tot. variable sampled every istep nodes (output_tot), shaped
        (nz, ny, nx); var: a name of OUTPUT_VARS, a moment name of MOMENTS,
        or the integer code"""
        if isinstance(var, str):
            var = self.OUTPUT_VARS[var] if var in self.OUTPUT_VARS else 16 + MOMENTS.index(var)
        dims = np.zeros(3, np.int32)
        self._check(self.lib.tg_output_dims(self.h, istep, dims.ctypes.data))
        out = np.zeros(int(dims.prod()), np.float32)
        self._check(self.lib.tg_output_var(self.h, int(var), istep, idx, idy, idz, out.ctypes.data))
        return out.reshape(dims[2], dims[1], dims[0])

    def output_particles(self, species: int, stride: int) -> dict:
        """output_tot's particle sample (prtl.tot) of one species: the
        particles with modulo(ind / 2, stride) = 0, device order"""
        cnt = ctypes.c_int64()
        self._check(self.lib.tg_output_particles(self.h, species, stride, 0, None, None, ctypes.byref(cnt)))
        cap = max(cnt.value, 1)
        vals = np.zeros((8, cap), np.float32)
        ids = np.zeros((2, cap), np.int32)
        self._check(self.lib.tg_output_particles(self.h, species, stride, cap, vals.ctypes.data, ids.ctypes.data,
                                                 ctypes.byref(cnt)))
        names = ("x", "y", "z", "u", "v", "w", "ch", "gamma")
        out = {k: vals[i, :cnt.value] for i, k in enumerate(names)}
        out["ind"], out["proc"] = ids[0, :cnt.value], ids[1, :cnt.value]
        return out

    def spectrum_x(self, gambins: int = 200) -> dict:
        """lab-frame and flow-frame energy spectra per x slice, divided by
        gamma - 1 (save_spectrum)"""
        nb = ctypes.c_int32()
        self._check(self.lib.tg_spectrum_x_bins(self.h, ctypes.byref(nb)))
        out = {k: np.zeros((gambins, nb.value), np.float32) for k in ("ions", "lecs", "ions_rest", "lecs_rest")}
        xg = np.zeros(gambins, np.float32)
        xs = np.zeros(nb.value, np.float32)
        gr = np.zeros(2, np.float32)
        self._check(self.lib.tg_spectrum_x(self.h, gambins, out["ions"].ctypes.data, out["lecs"].ctypes.data,
                                           out["ions_rest"].ctypes.data, out["lecs_rest"].ctypes.data,
                                           xg.ctypes.data, xs.ctypes.data, gr.ctypes.data))
        return dict(out, xgamma=xg, xslice=xs, gammin=float(gr[0]), gammax=float(gr[1]))

    # -- restart files (write_restart / restart) -------------------------------
    def write_restart(self, fields_path: str, particles_path: str, **meta) -> None:
        m = tg_restart_meta()
        for k, v in meta.items():
            setattr(m, k, v)
        self._check(self.lib.tg_write_restart(self.h, fields_path.encode(), particles_path.encode(),
                                              ctypes.byref(m)))

    def read_restart(self, fields_path: str, particles_path: str) -> dict:
        m = tg_restart_meta()
        self._check(self.lib.tg_read_restart(self.h, fields_path.encode(), particles_path.encode(),
                                             ctypes.byref(m)))
        return {k: getattr(m, k) for k, _ in tg_restart_meta._fields_}


def _diag_dict(d: tg_diag) -> dict:
    out = {k: getattr(d, k) for k, _ in tg_diag._fields_}
    out["p_part"] = list(d.p_part)
    out["p_field"] = list(d.p_field)
    return out


class EnsembleSim:
    """Many independent periodic 2D boxes stepped together (tg_ens_*): one
    launch per phase for all boxes. Each box keeps its own host arrays, laid
    out as for GpuSim; ``pinned`` page-locks them."""

    def __init__(self, cfgs, device: int = 0, pinned: bool = False):
        self.cfgs = list(cfgs)
        self.lib = load_library()
        n = len(self.cfgs)
        self.tcfgs = (tg_config * n)(*[make_tg_config(c, device) for c in self.cfgs])
        h = ctypes.c_void_p()
        rc = self.lib.tg_ens_init(self.tcfgs, n, ctypes.byref(h))
        if rc != TG_OK:
            raise TristanGpuError(rc, self.lib.tg_ens_last_error(None).decode())
        self.h = h
        self.fields, self.p, self._ions, self._lecs, self._pinned = [], [], [], [], []
        for b, c in enumerate(self.cfgs):
            lot = c.mx * c.my * c.mz
            self.fields.append({k: np.zeros(lot, np.float32) for k in FIELD_NAMES})
            self.p.append(np.zeros(2 * c.maxhlf, PARTICLE_DTYPE))
            self._ions.append(ctypes.c_int32(0))
            self._lecs.append(ctypes.c_int32(0))
            if pinned:
                rt = _cudart_lib()
                for arr in [self.p[b]] + [self.fields[b][k] for k in FIELD_NAMES]:
                    if rt.cudaHostRegister(arr.ctypes.data, arr.nbytes, 0) != 0:
                        raise TristanGpuError(TG_ERR_CUDA, "cudaHostRegister failed")
                    self._pinned.append(arr)
            self._check(self.lib.tg_ens_bind_fields(self.h, b, *[self.fields[b][k].ctypes.data
                                                                 for k in FIELD_NAMES]))
            self._check(self.lib.tg_ens_bind_particles(self.h, b, self.p[b].ctypes.data,
                                                       ctypes.addressof(self._ions[b]),
                                                       ctypes.addressof(self._lecs[b])))

    @property
    def nbox(self) -> int:
        return len(self.cfgs)

    def close(self):
        if getattr(self, "h", None):
            self.lib.tg_ens_finalize(self.h)
            self.h = None
            for arr in getattr(self, "_pinned", []):
                _cudart_lib().cudaHostUnregister(arr.ctypes.data)
            self._pinned = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != TG_OK:
            raise TristanGpuError(rc, self.lib.tg_ens_last_error(self.h).decode())

    def set_particles(self, box: int, ions: np.ndarray, lecs: np.ndarray) -> None:
        mh = self.cfgs[box].maxhlf
        if len(ions) > mh or len(lecs) > mh:
            raise TristanGpuError(TG_ERR_OVERFLOW, "particle count exceeds maxhlf")
        self.p[box][: len(ions)] = ions
        self.p[box][mh: mh + len(lecs)] = lecs
        self._ions[box].value, self._lecs[box].value = len(ions), len(lecs)

    def set_fields(self, box: int, **arrays) -> None:
        for k, v in arrays.items():
            self.fields[box][k][:] = np.asarray(v, np.float32).ravel()

    def sync_from_host(self, mask: int = SYNC_ALL) -> None:
        self._check(self.lib.tg_ens_sync_from_host(self.h, mask))

    def sync_to_host(self, mask: int = SYNC_ALL) -> None:
        self._check(self.lib.tg_ens_sync_to_host(self.h, mask))

    def host_bytes(self, mask: int) -> int:
        n = 0
        for b, c in enumerate(self.cfgs):
            per = c.mx * c.my * c.mz * 4
            n += per * 3 * sum(1 for m in (SYNC_E, SYNC_B, SYNC_CUR) if mask & m)
            if mask & SYNC_PARTICLES:
                n += (self._ions[b].value + self._lecs[b].value) * PARTICLE_DTYPE.itemsize
        return n

    def ions(self, box: int) -> np.ndarray:
        return self.p[box][: self._ions[box].value]

    def lecs(self, box: int) -> np.ndarray:
        mh = self.cfgs[box].maxhlf
        return self.p[box][mh: mh + self._lecs[box].value]

    def field(self, box: int, name: str) -> np.ndarray:
        c = self.cfgs[box]
        return self.fields[box][name].reshape(c.mz, c.my, c.mx)

    def counts(self, box: int):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.tg_ens_get_counts(self.h, box, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def step(self, n: int = 1):
        self._check(self.lib.tg_ens_step(self.h, int(n)))

    def step_timed(self, n: int) -> float:
        ms = ctypes.c_float()
        self._check(self.lib.tg_ens_step_timed(self.h, int(n), ctypes.byref(ms)))
        return float(ms.value)

    def synchronize(self):
        self._check(self.lib.tg_ens_synchronize(self.h))

    def kernels_per_step(self) -> int:
        return int(self.lib.tg_ens_kernels_per_step(self.h))

    def diagnostics(self, box: int) -> dict:
        d = tg_diag()
        self._check(self.lib.tg_ens_diag_fp64(self.h, box, ctypes.byref(d)))
        return _diag_dict(d)


def ensemble_autotune(cfgs, particles, laps: int = 2, device: int = 0):
    """One tile shape and sort cadence for all boxes (tg_ens_autotune),
    timed on `particles` = [(ions, lecs) per box]; updates every cfg in place
    and returns (best ms per lap, table)."""
    lib = load_library()
    n = len(cfgs)
    arrs, ni, nl = [], [], []
    for c, (ions, lecs) in zip(cfgs, particles):
        p = np.zeros(2 * c.maxhlf, PARTICLE_DTYPE)
        p[: len(ions)] = ions
        p[c.maxhlf: c.maxhlf + len(lecs)] = lecs
        arrs.append(p)
        ni.append(ctypes.c_int32(len(ions)))
        nl.append(ctypes.c_int32(len(lecs)))
    tc = (tg_config * n)(*[make_tg_config(c, device) for c in cfgs])
    pp = (ctypes.c_void_p * n)(*[a.ctypes.data for a in arrs])
    pi = (ctypes.c_void_p * n)(*[ctypes.addressof(x) for x in ni])
    pl = (ctypes.c_void_p * n)(*[ctypes.addressof(x) for x in nl])
    best = ctypes.c_float()
    table = np.zeros((64, 5), np.float32)
    rows = lib.tg_ens_autotune(tc, n, pp, pi, pl, int(laps), ctypes.byref(best), table.ctypes.data, 64)
    if rows < 0:
        raise TristanGpuError(-rows, "ensemble autotune: no candidate ran")
    for c, t in zip(cfgs, tc):
        c.tile = (int(t.tile[0]), int(t.tile[1]), int(t.tile[2]))
        c.sort_every = int(t.sort_every)
    return float(best.value), table[:rows]
