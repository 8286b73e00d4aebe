"""Restart files in the reference's format (write_restart / restart,
code/output.F90:2192-2218, code/restart.F90:209-255), gfortran unformatted
sequential records: the files decode with an independent record reader to
exactly the device state, records split into subrecords decode the same,
and a run resumed from the files continues bit for bit (fixed point) like
the uninterrupted run."""
import os

import numpy as np
import pytest

from fortran_records import parse_fields, parse_particles, read_records
from test_gpu_parity import assert_particles_equal, beams, random_fields, small_cfg

pytestmark = pytest.mark.gpu


def sim(cfg, ions=None, lecs=None, f=None):
    from tristan_gb300.gpu import GpuSim
    g = GpuSim(cfg)
    if f:
        g.set_fields(**f)
        g.sync_from_host()
    if ions is not None:
        g.set_particles(ions, lecs)
    return g


@pytest.mark.parametrize("max_sub", [0, 1000])
def test_restart_files_decode_to_the_device_state(tmp_path, max_sub):
    cfg = small_cfg(2, 3, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(5))
    g = sim(cfg, ions, lecs, f)
    g.step(3)
    fp, pp = str(tmp_path / "restflds.d"), str(tmp_path / "restprtl.d")
    g.write_restart(fp, pp, dseed=424242.0, lap=3, xinject=1.5, xinject2=2.5, xinject3=3.5, leftwall=20.0,
                    walloc=21.25, totalpartnum=7, max_subrecord=max_sub)
    g.sync_to_host()
    recs = read_records(fp)
    assert len(recs) == 1
    d = parse_fields(recs[0])
    assert d["dims"] == (cfg.mx, cfg.my, cfg.mz)
    for k in ("ex", "ey", "ez", "bx", "by", "bz"):
        np.testing.assert_array_equal(d["fields"][k], g.fields[k])
    assert (d["dseed"], d["lap"], d["xinject"], d["leftwall"], d["walloc"]) == (424242.0, 3, (1.5, 2.5, 3.5),
                                                                               20.0, 21.25)
    precs = read_records(pp)
    assert len(precs) == 1
    p = parse_particles(precs[0], g.p.dtype)
    assert p["maxhlf"] == cfg.maxhlf and p["totalpartnum"] == 7
    assert_particles_equal(p["ions"], g.ions)
    assert_particles_equal(p["lecs"], g.lecs)
    if max_sub:
        raw = open(pp, "rb").read()
        assert len(raw) > 8 + (20 + 40 * (len(g.ions) + len(g.lecs)))  # several subrecords
    g.close()


def test_resume_from_restart_is_bit_exact(tmp_path):
    cfg = small_cfg(2, 2, fixed=1, sort_every=2)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(6))
    a = sim(cfg, ions, lecs, f)
    a.step(4)
    fp, pp = str(tmp_path / "f.d"), str(tmp_path / "p.d")
    a.write_restart(fp, pp, dseed=1.0, lap=4)
    a.step(5)
    a.sync_to_host()
    b = sim(cfg)
    meta = b.read_restart(fp, pp)
    assert meta["lap"] == 4
    # currents are not in the files: the next lap recomputes them
    b.step(5)
    b.sync_to_host()
    for k in ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz"):
        np.testing.assert_array_equal(b.fields[k], a.fields[k], err_msg=k)
    assert_particles_equal(b.ions, a.ions)
    assert_particles_equal(b.lecs, a.lecs)
    a.close()
    b.close()
