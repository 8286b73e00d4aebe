"""A compiled host (tests/harness/mainloop.cpp) drives the C-ABI as the
reference's main loop would through its bind(C) shim: the state lives in
host arrays the caller owns, each lap is the sequence of per-subroutine
calls of code/tristanmainloop.F90:117-303 (or one tg_step_host call), and
the arrays come back at the end.

Bars: the harness builds and links against the library with the public
header alone (CPU); on the GPU, in fixed-point mode, the host arrays after
the laps equal the oracle's bit for bit (particles keyed by ind), for both
the per-subroutine and the one-call forms."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "harness", "mainloop.cpp")
LIB = os.path.join(ROOT, "tristan-mp-pu-master_densdecomp_gb300", "lib")


def build_harness(out_dir):
    exe = os.path.join(out_dir, "mainloop")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-L", LIB,
                    "-ltristan_gpu", "-Wl,-rpath," + LIB, "-o", exe], check=True, capture_output=True)
    return exe


def have_library():
    return os.path.exists(os.path.join(LIB, "libtristan_gpu.so"))


def test_harness_builds_and_links(tmp_path):
    if not have_library():
        pytest.skip("libtristan_gpu.so not built")
    exe = build_harness(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr


def write_state(path, cfg, fields, ions, lecs):
    from tristan_gb300.gpu import FIELD_NAMES, make_tg_config
    p = np.zeros(2 * cfg.maxhlf, setups.PARTICLE_DTYPE)
    p[: len(ions)] = ions
    p[cfg.maxhlf: cfg.maxhlf + len(lecs)] = lecs
    with open(path, "wb") as f:
        f.write(bytes(make_tg_config(cfg)))
        for k in FIELD_NAMES:
            f.write(np.ascontiguousarray(fields[k], np.float32).tobytes())
        f.write(p.tobytes())
        f.write(np.array([len(ions), len(lecs)], np.int32).tobytes())


def read_state(path, cfg):
    from tristan_gb300.gpu import FIELD_NAMES, tg_config
    import ctypes
    raw = open(path, "rb").read()
    off = ctypes.sizeof(tg_config)
    lot = cfg.mx * cfg.my * cfg.mz
    fields = {}
    for k in FIELD_NAMES:
        fields[k] = np.frombuffer(raw, np.float32, lot, off)
        off += 4 * lot
    p = np.frombuffer(raw, setups.PARTICLE_DTYPE, 2 * cfg.maxhlf, off)
    off += p.nbytes
    ni, ne = np.frombuffer(raw, np.int32, 2, off)
    return fields, p[:ni], p[cfg.maxhlf: cfg.maxhlf + ne]


@pytest.mark.gpu
@pytest.mark.parametrize("dims,order", [(2, 3), (3, 2)])
@pytest.mark.parametrize("form", ["subroutines", "fused"])
def test_harness_mainloop_bit_exact(tmp_path, dims, order, form):
    from test_gpu_parity import assert_particles_equal, beams, random_fields, small_cfg
    from tristan_gb300.gpu import FIELD_NAMES
    cfg = small_cfg(dims, order, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(31), scale=0.02)
    fields = {k: f.get(k, np.zeros(cfg.mx * cfg.my * cfg.mz, np.float32)) for k in FIELD_NAMES}
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_state(src, cfg, fields, ions, lecs)
    exe = build_harness(str(tmp_path))
    laps = 4
    args = [exe, src, dst, str(laps)] + (["fused"] if form == "fused" else [])
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    gf, gi, ge = read_state(dst, cfg)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs)
    o.step(laps)
    for k in FIELD_NAMES:
        np.testing.assert_array_equal(gf[k], o.fields[k], err_msg=k)
    assert_particles_equal(gi, o.ions)
    assert_particles_equal(ge, o.lecs)
