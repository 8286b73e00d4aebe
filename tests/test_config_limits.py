"""Argument checks of tg_init that run before any CUDA call (so they run on
CPU), and the layout of every public struct: the ctypes mirrors agree with
what a C compiler makes of include/tristan_gpu.h."""
import ctypes
import os
import shutil
import subprocess

import pytest

from tristan_gb300 import gpu
from tristan_gb300.config import SimConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def init_rc(cfg, **patch):
    lib = gpu.load_library()
    c = gpu.make_tg_config(cfg)
    for k, v in patch.items():
        setattr(c, k, v)
    h = ctypes.c_void_p()
    rc = lib.tg_init(ctypes.byref(c), ctypes.byref(h))
    return rc, lib.tg_last_error(None).decode()


@pytest.fixture(scope="module", autouse=True)
def need_library():
    if not os.path.exists(gpu.LIB_PATH):
        pytest.skip("library not built")


BASE = dict(dims=2, order=3, nx=32, ny=32, maxhlf=1024)


@pytest.mark.parametrize("patch,needle", [
    (dict(order=4), "order"),
    (dict(nghost=5), "nghost"),
    (dict(mz=3), "mz = 1"),
    (dict(mx=8, my=8), "too small"),
    (dict(my=3 + 7), "too small"),  # 3 interior rows: the images of ghost rows are ghost rows
    (dict(maxhlf=0), "maxhlf"),
    (dict(dims=4), "dims"),
])
def test_init_rejects_bad_configurations(patch, needle):
    rc, msg = init_rc(SimConfig(**{k: v for k, v in BASE.items() if k != "maxhlf"}, maxhlf=1024), **patch)
    assert rc == gpu.TG_ERR_ARG and needle in msg


def test_init_rejects_grids_beyond_int32_cell_indices():
    cfg = SimConfig(dims=3, order=2, nx=1300, ny=1300, nz=1300, maxhlf=1024)
    rc, msg = init_rc(cfg)
    assert rc == gpu.TG_ERR_ARG and "int32" in msg


def test_init_rejects_windows_beyond_shared_memory():
    cfg = SimConfig(dims=3, order=3, nx=64, ny=64, nz=64, maxhlf=1024, tile=(32, 32, 32))
    rc, msg = init_rc(cfg)
    assert rc == gpu.TG_ERR_ARG and "shared memory" in msg


C_LAYOUT = r'''
#include <stddef.h>
#include <stdio.h>
#include "tristan_gpu.h"
#define P(T, F) printf(#T "." #F " %zu\n", offsetof(T, F))
int main(void) {
    printf("tg_config %zu\n", sizeof(tg_config));
    printf("tg_diag %zu\n", sizeof(tg_diag));
    printf("tg_shock %zu\n", sizeof(tg_shock));
    printf("tg_restart_meta %zu\n", sizeof(tg_restart_meta));
    P(tg_config, x1in); P(tg_config, maxhlf); P(tg_config, diag_every);
    P(tg_shock, walloc); P(tg_shock, edge); P(tg_shock, xinject2); P(tg_shock, xinj_max); P(tg_shock, dseed);
    P(tg_shock, totalpartnum);
    P(tg_restart_meta, lap); P(tg_restart_meta, walloc); P(tg_restart_meta, max_subrecord);
    return 0;
}
'''


def test_struct_layouts_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(C_LAYOUT)
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)]).decode().splitlines())
    got = {k: int(v) for k, v in got.items()}
    mirrors = {"tg_config": gpu.tg_config, "tg_diag": gpu.tg_diag, "tg_shock": gpu.tg_shock,
               "tg_restart_meta": gpu.tg_restart_meta}
    for name, cls in mirrors.items():
        assert got[name] == ctypes.sizeof(cls), name
    for key, off in got.items():
        if "." in key:
            t, f = key.split(".")
            assert getattr(mirrors[t], f).offset == off, key


def test_init_counts_the_2d_field_copy_in_shared_memory():
    # 2D tiles carry the deposit window and a copy of the six field arrays
    # over the same cells: a 72 x 72 order-3 tile (77 x 77 window cells,
    # 142 KB each) fits one but not both in the 227 KB of a CTA
    cfg = SimConfig(dims=2, order=3, nx=144, ny=144, maxhlf=1024, tile=(72, 72, 1), sort_every=1)
    rc, msg = init_rc(cfg)
    assert rc == gpu.TG_ERR_ARG and "shared memory" in msg and "field copy" in msg


def test_init_drops_the_3d_field_copy_rather_than_refusing():
    # a 3D tile keeps its shared field copy only while two CTAs per SM fit
    # beside the deposit window; when they would not (here the drift of a
    # sort every second lap widens both), the copy is left out and the
    # geometry stands (on a host without a GPU tg_init then stops at the
    # device, past every argument check)
    cfg = SimConfig(dims=3, order=2, nx=64, ny=64, nz=64, maxhlf=1024, tile=(16, 8, 4), sort_every=2)
    rc, msg = init_rc(cfg)
    assert rc != gpu.TG_ERR_ARG, msg
