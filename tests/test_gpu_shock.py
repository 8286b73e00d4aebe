"""Collisionless-shock hooks on the GPU against the oracle's restatement of
user_pu/user_shock_pu.F90 (left wall with zigzag partial deposits,
conductor and right-edge field reset, moving injector with the reference's
random stream).

Bars: in fixed-point mode every field, every particle (keyed by ind), the
particle counts, the injector / wall positions and the generator state are
bit-exact after the initial load and after whole laps, through the fused
lap and through the per-subroutine entry points; the jump-ahead injection
stays exact when a gamma draw is redrawn (a seed is chosen so that a given
pair's draw comes out as 1.0); in FP32 mode the fields stay within the FP32
bounds of the parity tests.
"""
import numpy as np
import pytest

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

from test_gpu_parity import assert_fields_close, assert_particles_equal

pytestmark = pytest.mark.gpu

NAMES = ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz")
M = 2147483647


def shock_cfg(fixed, **kw):
    base = dict(dims=2, order=3, nx=96, ny=16, c=0.45, c_omp=4.0, ppc0=4.0, gamma0=15.0, delgam=1e-4,
                sigma=0.1, ntimes=4, corr=1.0, periodic=(0, 1, 1), fixed=fixed)
    base.update(kw)
    return SimConfig(**base)


def pair(cfg, laps, dseed=123457.0, region=None):
    from tristan_gb300.gpu import GpuSim
    sh, f, reg = setups.shock_params(cfg, dseed=dseed)
    reg = region or reg
    cfg.maxhlf = setups.shock_capacity(cfg, laps, sh) + int(0.5 * reg[4] * (reg[1] - reg[0] + 1) *
                                                           (reg[3] - reg[2] + 1))
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.shock_init(sh)
    o.inject_region(*reg)
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.shock_init(sh)
    g.inject_region(*reg)
    return o, g


def assert_state(o, g):
    s = g.shock_state()
    assert s["dseed"] == o.shock.dseed
    assert s["totalpartnum"] == o.shock.totalpartnum
    assert s["xinject2"] == o.shock.xinject2
    assert s["walloc"] == o.shock.walloc
    assert s["betainj"] == np.float32(o.shock.betainj)


def compare(o, g, names=NAMES):
    g.sync_to_host()
    for k in names:
        np.testing.assert_array_equal(g.fields[k], o.fields[k], err_msg=k)
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    assert_state(o, g)


def test_shock_initial_load_bit_exact():
    cfg = shock_cfg(1)
    o, g = pair(cfg, 2)
    assert o.st.ions == 976
    compare(o, g)
    g.close()


def test_shock_laps_fixed_point_bit_exact():
    cfg = shock_cfg(1)
    o, g = pair(cfg, 40)
    g.step(40)
    o.step_shock(40)
    compare(o, g)
    assert o.st.ions > 976 + 40 * 28  # injector ran every lap
    assert (o.ions["u"] > 0).sum() > 100  # the wall reflected particles
    g.close()


def test_shock_subroutines_bit_exact():
    cfg = shock_cfg(1)
    o, g = pair(cfg, 6)
    for _ in range(6):
        g.bc_b1(); g.bc_e1(); g.advance_Bhalfstep(); g.bc_b1()
        g.move_particles()
        g.advance_Bhalfstep(); g.bc_b1(); g.bc_b1()
        g.field_bc_user(); g.advance_Efield(); g.field_bc_user(); g.bc_e1(); g.field_bc_user()
        g.reset_currents(); g.particle_bc_user(); g.bc_e1(); g.bc_b1()
        g.deposit_particles(); g.exchange_current(); g.apply_filter1_opt(); g.add_current()
        g.field_bc_user(); g.inject_particles_user()
    o.step_shock(6)
    compare(o, g)
    g.close()


def seed_for_redraw(pair_index, electron=False):
    """initial seed whose gamma draw of the given pair returns
    (2^31 - 2) / 2^31, which rounds to 1.0 in single precision"""
    d = 13 * pair_index + (9 if electron else 4)
    return float((M - 1) * pow(16807, -d, M) % M)


@pytest.mark.parametrize("where", [10, 7000])
def test_shock_injection_with_gamma_redraw(where):
    """a redraw early (the host re-runs the parallel pass after it) and
    late (the finishing kernel draws the rest in sequence)"""
    cfg = shock_cfg(1, nx=96, ny=32, ppc0=8.0)
    region = (20.0, 80.0, 3.0, 35.0, 8.0, 1.0)  # 4 x 31 x 60 = 7440 pairs
    o, g = pair(cfg, 2, dseed=seed_for_redraw(where, electron=(where == 7000)), region=region)
    assert o.st.ions == 7440
    compare(o, g)
    g.close()


def test_shock_fp32_within_tolerance():
    cfg = shock_cfg(0)
    o, g = pair(cfg, 20)
    g.step(20)
    o.step_shock(20)
    g.sync_to_host()
    assert_fields_close(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    assert len(g.ions) == len(o.ions) and len(g.lecs) == len(o.lecs)
    assert_state(o, g)
    g.close()


@pytest.mark.parametrize("sort_every,laps", [(3, 41), (4, 17)])
def test_shock_sorted_every_few_laps_bit_exact(sort_every, laps):
    """between tile sorts the injected particles sit past the tile ranges
    and are moved by the tail kernel; the result does not depend on the
    cadence, also when the run stops between two sorts"""
    cfg = shock_cfg(1, sort_every=sort_every)
    o, g = pair(cfg, laps)
    g.step(laps)
    o.step_shock(laps)
    compare(o, g)
    g.close()


def test_shock_sorted_every_few_laps_diag_sorts_first():
    """an explicit diagnostic between sorts counts the injected tail"""
    from tristan_gb300.gpu import GpuSim, TristanGpuError
    a, b = shock_cfg(1, sort_every=3), shock_cfg(1, sort_every=1)
    _, ga = pair(a, 5)
    _, gb = pair(b, 5)
    ga.step(5)
    gb.step(5)
    da, db = ga.diagnostics(), gb.diagnostics()
    # FP64 sums whose order follows the tile contents
    assert da["charge_total"] == pytest.approx(db["charge_total"], rel=1e-12, abs=1e-9)
    for k in ("e_kin_ions", "e_kin_lecs"):  # per-thread FP32 partial sums
        assert da[k] == pytest.approx(db[k], rel=1e-6), k
    ga.close()
    gb.close()
    # the per-lap diagnostics walk tiles: refused together with the tail
    c = shock_cfg(1, sort_every=3, diag_every=1)
    sh, f, _ = setups.shock_params(c)
    c.maxhlf = 100000
    g = GpuSim(c)
    with pytest.raises(TristanGpuError):
        g.shock_init(sh)
    g.close()
