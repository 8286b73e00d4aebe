"""GPU parity: every phase of the C-ABI against the CPU oracle.

Bars (the oracle restates the reference Fortran in its operation order):
  * field phases (ghost copies, B/E advance, fold, filter, add_current),
    the mover and the periodic wrap: bit-exact;
  * the deposit in int64 fixed-point mode: bit-exact (integer accumulation
    is order independent, both sides round each contribution identically);
  * the deposit in FP32 mode: ||gpu - oracle||_2 <= 1e-5 ||oracle||_2 per
    component and every element within 1e-4 of the component's maximum
    (atomics change only the summation order);
  * whole laps in fixed-point mode: every field and particle bit-exact;
    in FP32 mode: fields within the same FP32 bounds after 20 laps.
Particles are compared keyed by `ind` (the device keeps them tile-sorted).
"""
import numpy as np
import pytest

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

pytestmark = pytest.mark.gpu

CASES = [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 3)]
FP32_TOL = 1e-5


def small_cfg(dims, order, **kw):
    base = dict(dims=dims, order=order, c=0.45, c_omp=4.0, gamma0=3.0, delgam=0.01, ntimes=3)
    if dims == 2:
        base.update(nx=40, ny=24, ppc0=8.0)
    else:
        base.update(nx=12, ny=10, nz=12, ppc0=4.0)
    base.update(kw)
    return SimConfig(**base)


def gpu_sim(cfg):
    from tristan_gb300.gpu import GpuSim
    return GpuSim(cfg)


def beams(cfg, seed=7):
    ions, lecs = setups.load_beams(cfg, seed=seed)
    setups.with_capacity(cfg, len(ions), len(lecs))
    return ions, lecs


def random_fields(cfg, rng, scale=0.02, names=("ex", "ey", "ez", "bx", "by", "bz")):
    return {k: (rng.standard_normal(cfg.ncells) * scale).astype(np.float32) for k in names}


def pair(cfg, ions=None, lecs=None, fields=None):
    """oracle and GPU domains with identical state"""
    o = oracle.OracleSim(cfg)
    g = gpu_sim(cfg)
    if fields:
        for k, v in fields.items():
            o.fields[k][:] = v
        g.set_fields(**fields)
        g.sync_from_host()
    if ions is not None:
        o.set_particles(ions, lecs)
        g.set_particles(ions, lecs)
    return o, g


def by_ind(p):
    return np.sort(p, order="ind")


def assert_particles_equal(a, b):
    assert len(a) == len(b)
    a, b = by_ind(a), by_ind(b)
    for k in ("x", "y", "z", "u", "v", "w", "ch", "ind", "proc", "splitlev"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def assert_fields_equal(o, g, names):
    for k in names:
        np.testing.assert_array_equal(g.fields[k], o.fields[k], err_msg=k)


def assert_fields_close(o, g, names, tol=FP32_TOL):
    """FP32 agreement: norm-wise relative error <= tol, and no element off by
    more than 10*tol of the array maximum (cells whose partial sums cancel
    carry ~100 ulp of summation-order noise)"""
    for k in names:
        ref = o.fields[k].astype(np.float64)
        got = g.fields[k].astype(np.float64)
        nrm = max(np.linalg.norm(ref), 1e-300)
        rel = np.linalg.norm(got - ref) / nrm
        assert rel <= tol, f"{k}: norm-wise relative error {rel:.3e} > {tol}"
        scale = max(np.abs(ref).max(), 1e-30)
        err = np.abs(got - ref).max()
        assert err <= 10 * tol * scale, f"{k}: max err {err:.3e} > {10 * tol} * {scale:.3e}"


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("dims,order", CASES)
def test_field_phases_bit_exact(dims, order):
    cfg = small_cfg(dims, order, maxhlf=16)
    rng = np.random.default_rng(1)
    f = random_fields(cfg, rng, names=("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz"))
    o, g = pair(cfg, fields=f)
    for name, oc in (("bc_b1", "to_bc_b1"), ("bc_e1", "to_bc_e1"), ("advance_Bhalfstep", "to_advance_b_halfstep"),
                     ("advance_Efield", "to_advance_e_fullstep"), ("add_current", "to_add_current")):
        getattr(g, name)()
        o.call(oc)
        g.sync_to_host()
        assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz"))
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
@pytest.mark.parametrize("q5", [False, True])
def test_fold_bit_exact(dims, order, q5):
    cfg = small_cfg(dims, order, maxhlf=16, quirks=oracle.QUIRK_Q5_LHS if q5 else 0)
    f = random_fields(cfg, np.random.default_rng(2), names=("curx", "cury", "curz"))
    o, g = pair(cfg, fields=f)
    g.exchange_current()
    o.call("to_exchange_current")
    g.sync_to_host()
    assert_fields_equal(o, g, ("curx", "cury", "curz"))
    g.close()


# thin local grids: fewer interior cells than ghost cells along an axis, so
# the fold's two target slabs overlap and are added in order, as the
# reference does (code/fieldboundaries.F90:1797-1812); the smallest is
# nghost/2 + 1 cells
THIN = [(2, 3, dict(nx=64, ny=4)), (2, 1, dict(nx=40, ny=3)), (2, 2, dict(nx=5, ny=24)),
        (3, 2, dict(nx=12, ny=4, nz=10)), (3, 3, dict(nx=10, ny=10, nz=4))]


@pytest.mark.parametrize("dims,order,grid", THIN)
@pytest.mark.parametrize("q5", [False, True])
def test_fold_thin_grids_bit_exact(dims, order, grid, q5):
    cfg = small_cfg(dims, order, maxhlf=16, quirks=oracle.QUIRK_Q5_LHS if q5 else 0, **grid)
    f = random_fields(cfg, np.random.default_rng(21), names=("curx", "cury", "curz"))
    o, g = pair(cfg, fields=f)
    g.exchange_current()
    o.call("to_exchange_current")
    g.sync_to_host()
    assert_fields_equal(o, g, ("curx", "cury", "curz"))
    g.close()


@pytest.mark.parametrize("dims,order,grid", THIN)
def test_laps_thin_grids_fixed_point_bit_exact(dims, order, grid):
    """whole laps on thin grids (the 64 x 4 order-3 box among them): every
    field and particle bit-exact in fixed point"""
    cfg = small_cfg(dims, order, fixed=1, **grid)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(22), scale=0.02)
    o, g = pair(cfg, ions, lecs, f)
    g.step(8)
    o.step(8)
    g.sync_to_host()
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz"))
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
@pytest.mark.parametrize("ntimes", [3, 4])
def test_filter_bit_exact(dims, order, ntimes):
    cfg = small_cfg(dims, order, maxhlf=16, ntimes=ntimes)
    f = random_fields(cfg, np.random.default_rng(3), names=("curx", "cury", "curz"))
    o, g = pair(cfg, fields=f)
    g.apply_filter1_opt()
    o.call("to_apply_filter1_opt")
    g.sync_to_host()
    assert_fields_equal(o, g, ("curx", "cury", "curz"))
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
def test_mover_bit_exact(dims, order):
    cfg = small_cfg(dims, order)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(4), scale=0.05)
    o, g = pair(cfg, ions, lecs, f)
    g.move_particles()
    o.call("to_move_particles")
    g.sync_to_host()
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
@pytest.mark.parametrize("fixed", [True, False])
def test_deposit(dims, order, fixed):
    cfg = small_cfg(dims, order, fixed=int(fixed))
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(5), scale=0.05)
    o, g = pair(cfg, ions, lecs, f)
    # move first (oracle), so positions carry displacements and some leave the box
    o.call("to_move_particles")
    g.set_particles(o.ions.copy(), o.lecs.copy())
    o.call("to_reset_currents")
    g.reset_currents()
    o.call("to_deposit_particles")
    g.deposit_particles()
    g.sync_to_host()
    if fixed:
        assert_fields_equal(o, g, ("curx", "cury", "curz"))
    else:
        assert_fields_close(o, g, ("curx", "cury", "curz"))
    assert np.abs(o.fields["curx"]).max() > 0
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
def test_reorder_matches_reference_order(dims, order):
    cfg = small_cfg(dims, order)
    ions, lecs = beams(cfg)
    rng = np.random.default_rng(6)
    perm_i, perm_l = rng.permutation(len(ions)), rng.permutation(len(lecs))
    ions, lecs = ions[perm_i], lecs[perm_l]
    o, g = pair(cfg, ions, lecs)
    # GPU sorts into tiles on upload; download gives the tile order, so
    # replay the reorder on the oracle from that same order
    g.sync_to_host()
    o.set_particles(g.ions.copy(), g.lecs.copy())
    g.reorder_particles(lap=10, force=True)
    o.call("to_reorder_particles_")
    g.sync_to_host()
    np.testing.assert_array_equal(g.ions, o.ions)
    np.testing.assert_array_equal(g.lecs, o.lecs)
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
def test_laps_fixed_point_bit_exact(dims, order):
    cfg = small_cfg(dims, order, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(8), scale=0.02)
    o, g = pair(cfg, ions, lecs, f)
    nlaps = 6
    g.step(nlaps)
    o.step(nlaps)
    g.sync_to_host()
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz", "curx", "cury", "curz"))
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    g.close()


@pytest.mark.parametrize("dims,order", CASES)
def test_laps_fp32_within_tolerance(dims, order):
    cfg = small_cfg(dims, order, fixed=0)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(9), scale=0.02)
    o, g = pair(cfg, ions, lecs, f)
    g.step(20)
    o.step(20)
    g.sync_to_host()
    assert_fields_close(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    assert len(g.ions) == len(o.ions) and len(g.lecs) == len(o.lecs)
    g.close()


@pytest.mark.parametrize("sort_every", [2, 3])
def test_sort_cadence_and_graph_replay(sort_every):
    """laps replayed from the captured graph (sort every k laps, windows
    widened for the drift) stay bit-exact in fixed-point mode"""
    cfg = small_cfg(2, 3, fixed=1, sort_every=sort_every)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(10), scale=0.02)
    o, g = pair(cfg, ions, lecs, f)
    g.step(2 * sort_every + 1)
    g.step(2 * sort_every)
    o.step(4 * sort_every + 1)
    g.sync_to_host()
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    assert_particles_equal(g.ions, o.ions)
    g.close()


def test_one_species_empty():
    cfg = small_cfg(2, 1, fixed=1)
    ions, lecs = beams(cfg)
    o, g = pair(cfg, ions, lecs[:0])
    g.step(3)
    o.step(3)
    g.sync_to_host()
    assert len(g.lecs) == 0
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    assert_particles_equal(g.ions, o.ions)
    g.close()


def test_small_tiles_force_global_fallback():
    """tiles of 4 cells with a relativistic beam: many deposits fall outside
    the window after the drift and take the global-atomic path"""
    cfg = small_cfg(2, 3, fixed=1, tile=(4, 4, 0), sort_every=4)
    ions, lecs = beams(cfg)
    o, g = pair(cfg, ions, lecs)
    g.step(8)
    o.step(8)
    g.sync_to_host()
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    g.close()


def test_autotune_picks_a_runnable_layout_that_stays_exact():
    from tristan_gb300.gpu import autotune
    cfg = small_cfg(2, 3, fixed=1)
    ions, lecs = beams(cfg)
    best, table = autotune(cfg, ions, lecs, laps=1)
    assert best > 0 and len(table) >= 3
    assert cfg.sort_every in (1, 2, 3) and cfg.tile[0] > 0
    o, g = pair(cfg, ions, lecs)
    g.step(7)
    o.step(7)
    g.sync_to_host()
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    g.close()


@pytest.mark.parametrize("dims,order", [(2, 1), (2, 3), (3, 2)])
def test_open_x_boundary_discards_like_the_reference(dims, order):
    """x open (periodicx = 0): particles leaving [x1in, x2in] are discarded
    (deposit_particles' boundary loop); counts, survivors and fields match"""
    cfg = small_cfg(dims, order, fixed=1, periodic=(0, 1, 1))
    ions, lecs = beams(cfg)
    o, g = pair(cfg, ions, lecs)
    g.step(5)
    o.step(5)
    g.sync_to_host()
    ni, nl = g.counts()
    assert (ni, nl) == (o.st.ions, o.st.lecs)
    assert ni < len(ions)  # some left through the open faces
    assert_particles_equal(g.ions, o.ions)
    assert_particles_equal(g.lecs, o.lecs)
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    g.close()


def test_external_constant_field_in_mover():
    """get_external_fields hook: a constant external B in the mover"""
    cfg = small_cfg(2, 2, fixed=1, external_fields=1, ext=(0.0, 0.0, 0.0, 0.0, 0.0, 0.05))
    ions, lecs = beams(cfg)
    o, g = pair(cfg, ions, lecs)
    g.step(3)
    o.step(3)
    g.sync_to_host()
    assert_particles_equal(g.ions, o.ions)
    assert_fields_equal(o, g, ("ex", "ey", "ez", "bx", "by", "bz"))
    g.close()


def test_failure_detection_overflow_and_out_of_grid():
    """errors come back as status codes, never as a GPU fault: a species
    count above maxhlf is refused on upload, and a particle outside the grid
    is flagged by the device status word and dropped"""
    from tristan_gb300.gpu import TG_ERR_BOUNDS, TG_ERR_OVERFLOW, TristanGpuError
    cfg = small_cfg(2, 1, maxhlf=64)
    ions, lecs = setups.load_beams(cfg, seed=3)
    g = gpu_sim(cfg)
    with pytest.raises(TristanGpuError) as e:
        g._ions.value = cfg.maxhlf + 1
        g.sync_from_host(8)
    assert e.value.code == TG_ERR_OVERFLOW
    bad = ions[:8].copy()
    bad["x"][3] = -50.0  # outside the array
    g.set_particles(bad, lecs[:8], upload=False)
    g._ions.value, g._lecs.value = 8, 8
    g.sync_from_host(8)
    with pytest.raises(TristanGpuError) as e:
        g.synchronize()
    assert e.value.code == TG_ERR_BOUNDS
    g.synchronize()  # the status word was cleared with the report
    assert g.counts() == (7, 8)
    g.close()
