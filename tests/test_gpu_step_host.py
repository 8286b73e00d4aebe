"""tg_step_host: main-loop passes with the bound host arrays as the state
(per lap E, B and the particle records go up, the lap runs, E, B, the
currents, the records and the counts come back).

Bars: in fixed-point mode the overlapped form (page-locked records on an
all-periodic domain: each species' records move while the other species
and the field phases run) leaves the host fields and records bit-identical
to the oracle after whole laps, records compared as sets keyed by ind; the
sequential form (pageable records) gives the same; a record outside the
grid on the way up is dropped and reported, and the compacted records come
back."""
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


def test_step_host_drops_record_outside_grid():
    from tristan_gb300.gpu import TG_ERR_BOUNDS, TristanGpuError
    cfg = small_cfg(2, 1, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(23), scale=0.02)
    bad = ions.copy()
    bad["x"][3] = -50.0  # outside the array
    g = host_sim(cfg, bad, lecs, f, True)
    with pytest.raises(TristanGpuError) as e:
        g.step_host(1)
    assert e.value.code == TG_ERR_BOUNDS
    assert (len(g.ions), len(g.lecs)) == (len(ions) - 1, len(lecs))
    assert -50.0 not in set(g.ions["x"].tolist())
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
