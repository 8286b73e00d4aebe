"""Batched ensemble (tg_ens_*) against single-domain contexts.

Every box of an ensemble runs the single-domain path's arithmetic, so:
  * in fixed-point mode each box's fields and particles after several laps
    (graph-replayed cycles and single laps, sorts included) equal bit for
    bit those of a single-domain context of the same box, and, for one box,
    those of the CPU oracle;
  * in FP32 mode (float atomics, different tile grouping) each box stays
    within the FP32 bounds of the parity tests;
  * the FP64 diagnostics of a box match the single-domain ones (FP64 field
    and charge sums to 1e-12 relative; the kinetic energies, which sum
    FP32 per-thread partials, to 1e-6).
"""
import numpy as np
import pytest

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

from test_gpu_parity import (assert_fields_close, assert_particles_equal, random_fields)

pytestmark = pytest.mark.gpu

NAMES = ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz")


def small_ensemble(fixed, sort_every=2, orders=(1, 2, 3, 3, 1), seed=11,
                   field_names=("ex", "ey", "ez", "bx", "by", "bz")):
    cfgs, _ = setups.ensemble_configs(nbox=len(orders), seed=seed, sides=(24, 32, 40, 56),
                                      ppc_range=(2, 8), fixed=fixed, sort_every=sort_every)
    for c, o in zip(cfgs, orders):
        c.order = o
        c.c_omp = 4.0
        c.ntimes = 3
    parts = setups.load_ensemble(cfgs, seed=5)
    rng = np.random.default_rng(12)
    fields = [random_fields(c, rng, scale=0.02, names=field_names) for c in cfgs]
    return cfgs, parts, fields


def build(cfgs, parts, fields):
    from tristan_gb300.gpu import EnsembleSim
    e = EnsembleSim(cfgs)
    for b, ((ions, lecs), f) in enumerate(zip(parts, fields)):
        e.set_particles(b, ions, lecs)
        e.set_fields(b, **f)
    e.sync_from_host()
    return e


def single(cfg, ions, lecs, f):
    from tristan_gb300.gpu import GpuSim
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.set_particles(ions, lecs)
    return g


def test_ensemble_fixed_point_bit_exact_vs_single_domain():
    cfgs, parts, fields = small_ensemble(fixed=1)
    e = build(cfgs, parts, fields)
    nlaps = 7  # one graph cycle of 4 laps, then 3 single laps
    e.step(nlaps)
    e.sync_to_host()
    assert e.kernels_per_step() > 0
    for b, c in enumerate(cfgs):
        g = single(c, *parts[b], fields[b])
        g.step(nlaps)
        g.sync_to_host()
        for k in NAMES:
            np.testing.assert_array_equal(e.fields[b][k], g.fields[k], err_msg=f"box {b} {k}")
        assert_particles_equal(e.ions(b), g.ions)
        assert_particles_equal(e.lecs(b), g.lecs)
        assert e.counts(b) == (len(parts[b][0]), len(parts[b][1]))
        g.close()
    e.close()


def test_ensemble_box_matches_oracle():
    cfgs, parts, fields = small_ensemble(fixed=1, orders=(3, 2))
    e = build(cfgs, parts, fields)
    e.step(3)
    e.sync_to_host()
    for b in range(2):
        o = oracle.OracleSim(cfgs[b])
        for k, v in fields[b].items():
            o.fields[k][:] = v
        o.set_particles(*parts[b])
        o.step(3)
        for k in NAMES:
            np.testing.assert_array_equal(e.fields[b][k], o.fields[k], err_msg=f"box {b} {k}")
        assert_particles_equal(e.ions(b), o.ions)
        assert_particles_equal(e.lecs(b), o.lecs)
    e.close()


def test_ensemble_fp32_within_tolerance():
    cfgs, parts, fields = small_ensemble(fixed=0, sort_every=1)
    e = build(cfgs, parts, fields)
    e.step(10)
    e.sync_to_host()
    for b, c in enumerate(cfgs):
        o = oracle.OracleSim(c)
        for k, v in fields[b].items():
            o.fields[k][:] = v
        o.set_particles(*parts[b])
        o.step(10)

        class View:
            pass
        v = View()
        v.fields = e.fields[b]
        assert_fields_close(o, v, ("ex", "ey", "ez", "bx", "by", "bz"))
        assert len(e.ions(b)) == len(o.ions)
    e.close()


def test_ensemble_diagnostics_match_single_domain():
    # E starts at zero over a neutral plasma, so Gauss's law holds at lap 0
    # and the charge-conserving deposit keeps the residual at rounding level
    cfgs, parts, fields = small_ensemble(fixed=1, orders=(1, 3, 2), field_names=("bx", "by", "bz"))
    e = build(cfgs, parts, fields)
    e.step(4)
    for b, c in enumerate(cfgs):
        g = single(c, *parts[b], fields[b])
        g.step(4)
        de, dg = e.diagnostics(b), g.diagnostics()
        # fields and the fixed-point charge: FP64 sums, order noise only
        for k in ("gauss_residual", "charge_total", "e_field", "e_mag"):
            assert de[k] == pytest.approx(dg[k], rel=1e-12, abs=1e-300), (b, k)
        # kinetic energies: per-thread compensated FP32 partial sums, whose
        # grouping follows the (atomic) order of particles within a tile
        for k in ("e_kin_ions", "e_kin_lecs"):
            assert de[k] == pytest.approx(dg[k], rel=1e-6), (b, k)
        # against one species' charge density the reference arithmetic's
        # rounding floor is far below 1e-5
        ni, nl = len(parts[b][0]), len(parts[b][1])
        ncell = c.interior_cells
        norm_s = (abs(c.qi) * ni + abs(c.qe) * nl) / (2.0 * ncell) * np.sqrt(ncell)
        assert de["gauss_abs"] / norm_s <= 1e-5
        g.close()
    e.close()


def test_ensemble_autotune_and_uneven_sizes():
    from tristan_gb300.gpu import EnsembleSim, ensemble_autotune
    cfgs, parts, fields = small_ensemble(fixed=1, orders=(3, 1, 2))
    best, table = ensemble_autotune(cfgs, parts, laps=1)
    assert best > 0 and len(table) >= 1
    assert all(c.sort_every == cfgs[0].sort_every and c.tile == cfgs[0].tile for c in cfgs)
    e = build(cfgs, parts, fields)
    e.step(2 * cfgs[0].sort_every + 1)
    e.sync_to_host()
    for b, c in enumerate(cfgs):
        g = single(c, *parts[b], fields[b])
        g.step(2 * c.sort_every + 1)
        g.sync_to_host()
        for k in ("ex", "bz", "curx"):
            np.testing.assert_array_equal(e.fields[b][k], g.fields[k], err_msg=f"box {b} {k}")
        g.close()
    e.close()


def test_two_ensembles_share_the_constant_table_in_turn():
    """Ensembles of up to 72 boxes read their tile arguments from one
    constant-memory table per device; two ensembles stepped in turn on one
    device (each waits for the other's laps) stay bit-exact against
    single-domain contexts"""
    cfgs_a, parts_a, fields_a = small_ensemble(fixed=1, orders=(3, 1, 2), seed=11)
    cfgs_b, parts_b, fields_b = small_ensemble(fixed=1, orders=(2, 3), seed=12)
    ea = build(cfgs_a, parts_a, fields_a)
    eb = build(cfgs_b, parts_b, fields_b)
    for _ in range(3):
        ea.step(2)
        eb.step(3)
    ea.sync_to_host()
    eb.sync_to_host()
    for cfgs, parts, fields, e, laps in ((cfgs_a, parts_a, fields_a, ea, 6), (cfgs_b, parts_b, fields_b, eb, 9)):
        for b, c in enumerate(cfgs):
            g = single(c, *parts[b], fields[b])
            g.step(laps)
            g.sync_to_host()
            for k in ("ex", "bz", "curx", "cury"):
                np.testing.assert_array_equal(e.fields[b][k], g.fields[k], err_msg=f"box {b} {k}")
            assert_particles_equal(e.ions(b), g.ions)
            g.close()
    ea.close()
    eb.close()


def test_ensemble_beyond_the_constant_table_matches_single_domain():
    """73 boxes: more than the constant-memory table holds, so the tiles read
    their arguments from shared memory; still bit-exact per box"""
    orders = tuple(1 + (b % 3) for b in range(73))
    cfgs, _ = setups.ensemble_configs(nbox=73, seed=31, sides=(24, 32), ppc_range=(2, 4), fixed=1, sort_every=2)
    for c, o in zip(cfgs, orders):
        c.order = o
        c.c_omp = 4.0
        c.ntimes = 2
    parts = setups.load_ensemble(cfgs, seed=7)
    rng = np.random.default_rng(13)
    fields = [random_fields(c, rng, scale=0.02) for c in cfgs]
    e = build(cfgs, parts, fields)
    e.step(5)
    e.sync_to_host()
    for b in (0, 1, 2, 40, 72):
        g = single(cfgs[b], *parts[b], fields[b])
        g.step(5)
        g.sync_to_host()
        for k in ("ex", "bz", "curx"):
            np.testing.assert_array_equal(e.fields[b][k], g.fields[k], err_msg=f"box {b} {k}")
        assert_particles_equal(e.ions(b), g.ions)
        g.close()
    e.close()
