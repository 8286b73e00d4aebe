"""Edge cases of the host-facing entry points: empty species, samples that
select nothing, a sampling step larger than the grid, repeated host laps
with an empty species; every call returns a status, none faults."""
import numpy as np
import pytest

import oracle
from test_gpu_parity import assert_fields_equal, assert_particles_equal, beams, random_fields, small_cfg
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

pytestmark = pytest.mark.gpu

ALL = ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz")


def test_step_host_with_an_empty_species():
    from tristan_gb300.gpu import GpuSim
    cfg = small_cfg(2, 3, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(41), scale=0.02)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs[:0])
    g = GpuSim(cfg, pinned=True)
    g.set_fields(**f)
    g.set_particles(ions, lecs[:0], upload=False)
    g.step_host(3)
    o.step(3)
    assert len(g.lecs) == 0
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.ions, o.ions)
    g.close()


def test_output_samples_that_select_nothing():
    from tristan_gb300.gpu import GpuSim
    cfg = small_cfg(2, 1, fixed=1)
    ions, lecs = beams(cfg)
    g = GpuSim(cfg)
    g.set_particles(ions, lecs)
    g.step(1)
    # a sampling step beyond the grid leaves no node
    big = 10 * max(cfg.mx, cfg.my)
    out = g.output_var("ex", big)
    assert out.size == 0
    # a stride above every ind / 2 selects the particles with ind / 2 = 0 only
    s = g.output_particles(0, 10 ** 9)
    assert np.all(np.asarray(s["ind"]) // 2 == 0)
    g.close()
    # no particles at all: spectra and samples are empty, not errors
    g = GpuSim(cfg)
    g.set_particles(ions[:0], lecs[:0])
    assert g.output_particles(1, 1)["x"].size == 0
    sp = g.spectrum_x()  # gamma range [1, 1]: the reference's axis is not finite either
    assert sp["ions"].shape == sp["lecs"].shape == (200, sp["xslice"].size)
    assert g.output_var("tdens", 2).max() == 0.0
    g.close()


def test_bad_arguments_return_status():
    from tristan_gb300.gpu import GpuSim, TristanGpuError
    cfg = small_cfg(2, 1, fixed=1)
    ions, lecs = beams(cfg)
    g = GpuSim(cfg)
    g.set_particles(ions, lecs)
    for call in (lambda: g.output_var(99, 2), lambda: g.output_var("ex", 0), lambda: g.output_particles(2, 1),
                 lambda: g.output_particles(0, 0), lambda: g.spectrum_x(gambins=0)):
        with pytest.raises(TristanGpuError):
            call()
    g.step(1)  # the context stays usable
    g.sync_to_host()
    assert len(g.ions) == len(ions)
    g.close()


def test_phase_timers_follow_the_reference_timer_groups():
    """tg_phase_times splits a timed lap as the reference's per-lap timers
    (Field slv, Mover + Deposit, Currnt exch, Filter, Reorder): every phase
    that runs has a positive time"""
    from tristan_gb300.gpu import PHASES, GpuSim
    cfg = SimConfig(dims=2, order=3, nx=64, ny=48, ppc0=8.0, c_omp=4.0, ntimes=4, sort_every=1, diag_every=1)
    ions, lecs = setups.load_beams(cfg, seed=3)
    setups.with_capacity(cfg, len(ions), len(lecs))
    g = GpuSim(cfg)
    try:
        g.set_particles(ions, lecs)
        g.step(2)
        g.enable_timing(True)
        g.step_timed(4)
        ph = g.phase_times()
    finally:
        g.close()
    assert tuple(ph) == PHASES
    for k in PHASES:
        assert ph[k] > 0.0, (k, ph[k])
