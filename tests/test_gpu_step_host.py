"""tg_step_host: main-loop passes with the bound host arrays as the state
(per lap E, B and the particle records go up, the lap runs, E, B, the
currents, the records and the counts come back).

Bars: in fixed-point mode the overlapped form (page-locked records on an
all-periodic domain: each species' records move while the other species
and the field phases run) leaves the host fields and records bit-identical
to the oracle after whole laps, records compared as sets keyed by ind; the
sequential form (pageable records) gives the same, and so does the
overlapped form with each species in parts (the diagnostics' kinetic
energies and particle momenta, compensated FP32 partial sums grouped
differently, to 1e-6 of the kinetic energy); a record
outside the grid on the way up is dropped and reported, and the compacted
records come back."""
import numpy as np
import pytest

from test_gpu_parity import (assert_fields_equal, assert_particles_equal, beams, pair, random_fields,
                             small_cfg)

pytestmark = pytest.mark.gpu

ALL = ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz")


def host_sim(cfg, ions, lecs, fields, pinned):
    from tristan_gb300.gpu import GpuSim
    g = GpuSim(cfg, pinned=pinned)
    g.set_fields(**fields)
    g.set_particles(ions, lecs, upload=False)
    return g


@pytest.mark.parametrize("dims,order,sort_every,diag", [(2, 3, 1, 1), (2, 1, 2, 0), (3, 2, 1, 1)])
@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_bit_exact(dims, order, sort_every, diag, pinned):
    cfg = small_cfg(dims, order, fixed=1, sort_every=sort_every, diag_every=diag)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(21), scale=0.02)
    o, g0 = pair(cfg, ions, lecs, f)
    g0.close()
    g = host_sim(cfg, ions, lecs, f, pinned)
    nlaps = 5
    for _ in range(nlaps):
        g.step_host(1)
    o.step(nlaps)
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    # the device stays usable after host-driven laps: more laps from the graph
    g.step(2)
    o.step(2)
    g.sync_to_host()
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.ions, o.ions)
    g.close()


@pytest.mark.parametrize("dims,order,parts", [(2, 3, 2), (2, 2, 3), (3, 1, 4), (2, 1, 8)])
def test_step_host_in_parts_bit_exact(dims, order, parts):
    """each species in parts, each part sorted and pushed on its own: the
    same fields, records and FP64 diagnostics as the oracle, laps with the
    graph afterwards"""
    cfg = small_cfg(dims, order, fixed=1, sort_every=1, diag_every=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(25), scale=0.02)
    o, g0 = pair(cfg, ions, lecs, f)
    g0.step(3)
    h0 = g0.diag_history(3)
    g0.close()
    g = host_sim(cfg, ions, lecs, f, True)
    g.set_host_parts(parts)
    g.step_host(3)
    o.step(3)
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    # the diagnostics' particle pass ran part by part: the charge (fixed
    # point) and the field sums agree to FP64 order noise; kinetic energies
    # and particle momenta are per-thread compensated FP32 partial sums,
    # grouped differently when a tile's particles come in parts
    h = g.diag_history(3)
    assert h.shape == h0.shape == (3, 16)
    exact = [0, 1, 2, 3, 4, 10, 11, 12]
    np.testing.assert_allclose(h[:, exact], h0[:, exact], rtol=1e-12, atol=1e-12 * float(np.abs(h0).max()))
    scale = float(np.abs(h0[:, 5:7]).sum(axis=1).max())
    np.testing.assert_allclose(h[:, 5:10], h0[:, 5:10], rtol=0, atol=1e-6 * scale)
    g.step(2)
    o.step(2)
    g.sync_to_host()
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()


def test_step_host_parts_argument():
    from tristan_gb300.gpu import TG_ERR_ARG, TristanGpuError
    cfg = small_cfg(2, 1, fixed=1)
    ions, lecs = beams(cfg)
    g = host_sim(cfg, ions, lecs, random_fields(cfg, np.random.default_rng(26), scale=0.02), True)
    for bad in (-1, 9):
        with pytest.raises(TristanGpuError) as e:
            g.set_host_parts(bad)
        assert e.value.code == TG_ERR_ARG
    g.set_host_parts(0)
    g.close()


def test_step_host_host_edits_between_laps():
    """the host may change the records between passes (here: drops the last
    ten electrons and moves one ion): the next pass starts from them"""
    cfg = small_cfg(2, 2, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(22), scale=0.02)
    o, g0 = pair(cfg, ions, lecs, f)
    g0.close()
    g = host_sim(cfg, ions, lecs, f, True)
    g.step_host(2)
    o.step(2)
    ni, ne = len(g.ions), len(g.lecs)
    gi, ge = g.ions.copy(), g.lecs.copy()
    gi["x"][5] = np.float32(cfg.nx / 2 + 3.25)
    g.set_particles(gi, ge[: ne - 10], upload=False)
    oi, oe = o.ions.copy(), o.lecs.copy()
    k = np.nonzero(oi["ind"] == gi["ind"][5])[0][0]
    oi["x"][k] = gi["x"][5]
    drop = set(ge["ind"][ne - 10:].tolist())
    o.set_particles(oi, oe[[i not in drop for i in oe["ind"]]])
    g.step_host(2)
    o.step(2)
    assert (len(g.ions), len(g.lecs)) == (ni, ne - 10)
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()


@pytest.mark.parametrize("parts", [1, 3])
def test_step_host_drops_record_outside_grid(parts):
    from tristan_gb300.gpu import TG_ERR_BOUNDS, TristanGpuError
    cfg = small_cfg(2, 1, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(23), scale=0.02)
    bad = ions.copy()
    bad["x"][3] = -50.0  # outside the array
    bad["x"][len(bad) - 2] = -50.0  # in the last part
    g = host_sim(cfg, bad, lecs, f, True)
    g.set_host_parts(parts)
    with pytest.raises(TristanGpuError) as e:
        g.step_host(1)
    assert e.value.code == TG_ERR_BOUNDS
    assert (len(g.ions), len(g.lecs)) == (len(ions) - 2, len(lecs))
    assert -50.0 not in set(g.ions["x"].tolist())
    assert set(g.ions["ind"].tolist()) == set(ions["ind"].tolist()) - {ions["ind"][3], ions["ind"][len(ions) - 2]}
    g.step_host(1)  # the status word was cleared with the report
    g.close()


def test_pin_host_from_the_library():
    """tg_pin_host page-locks the bound arrays (the overlapped form then
    runs) and is harmless when repeated; results stay bit-exact"""
    cfg = small_cfg(2, 3, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(24), scale=0.02)
    o, g0 = pair(cfg, ions, lecs, f)
    g0.close()
    g = host_sim(cfg, ions, lecs, f, False)
    g.pin_host()
    g.pin_host()
    g.step_host(3)
    o.step(3)
    assert_fields_equal(o, g, ALL)
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()
