"""The C oracle against the independent pure-Python transliteration
(tests/golden/make_golden.py): every phase must agree bit for bit."""
import glob
import os

import numpy as np
import pytest

import oracle
from tristan_gb300.config import SimConfig

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "golden_*.npz")))


def make_sim(g, **kw):
    cfg = SimConfig(dims=int(g["dims"]), order=int(g["order"]), nx=int(g["nx"]), ny=int(g["ny"]),
                    nz=int(g["nz"]), c=float(g["c"]), corr=float(g["corr"]), ntimes=2,
                    maxhlf=256, **kw)
    sim = oracle.OracleSim(cfg)
    sim.st.qi = float(g["q"])
    sim.st.qe = -float(g["q"])
    return sim


def set_fields(sim, arrs, names):
    for a, n in zip(arrs, names):
        sim.fields[n][:] = a


@pytest.fixture(params=GOLDEN, ids=[os.path.basename(p)[7:-4] for p in GOLDEN])
def golden(request):
    return np.load(request.param)


def test_golden_present():
    assert len(GOLDEN) == 6


def test_mover(golden):
    sim = make_sim(golden)
    set_fields(sim, golden["fields"], ("ex", "ey", "ez", "bx", "by", "bz"))
    parts = golden["particles"]
    sim.set_particles(parts, parts[:0])
    sim.lib.to_mover(sim.ptr, 0, len(parts), float(golden["qm"]))
    got = sim.ions
    mv = golden["moved"]
    for col, k in enumerate(("x", "y", "z", "u", "v", "w")):
        np.testing.assert_array_equal(got[k], mv[:, col], err_msg=k)


def test_deposit_and_wrap(golden):
    sim = make_sim(golden)
    parts = golden["particles"].copy()
    mv = golden["moved"]
    for col, k in enumerate(("x", "y", "z", "u", "v", "w")):
        parts[k] = mv[:, col]
    sim.set_particles(parts, parts[:0])
    sim.call("to_reset_currents")
    sim.call("to_deposit_particles")
    for a, n in zip(golden["deposit"], ("curx", "cury", "curz")):
        np.testing.assert_array_equal(sim.fields[n], a, err_msg=n)
    got = np.sort(sim.ions, order="ind")
    assert len(got) == len(parts)
    w = golden["wrapped"]
    idx = np.argsort(parts["ind"])
    for col, k in enumerate(("x", "y", "z")):
        np.testing.assert_array_equal(got[k], w[idx, col], err_msg=k)


def test_advance_b(golden):
    sim = make_sim(golden)
    set_fields(sim, golden["fields"], ("ex", "ey", "ez", "bx", "by", "bz"))
    sim.call("to_advance_b_halfstep")
    for a, n in zip(golden["advance_b"], ("ex", "ey", "ez", "bx", "by", "bz")):
        np.testing.assert_array_equal(sim.fields[n], a, err_msg=n)


def test_advance_e(golden):
    sim = make_sim(golden)
    set_fields(sim, golden["fields"], ("ex", "ey", "ez", "bx", "by", "bz"))
    sim.call("to_advance_e_fullstep")
    for a, n in zip(golden["advance_e"], ("ex", "ey", "ez", "bx", "by", "bz")):
        np.testing.assert_array_equal(sim.fields[n], a, err_msg=n)


def test_ghost_copy(golden):
    sim = make_sim(golden)
    set_fields(sim, golden["fields"], ("ex", "ey", "ez", "bx", "by", "bz"))
    sim.call("to_bc_b1")
    for a, n in zip(golden["bc_b"], ("bx", "by", "bz")):
        np.testing.assert_array_equal(sim.fields[n], a, err_msg=n)


@pytest.mark.parametrize("q5", [False, True])
def test_fold(golden, q5):
    sim = make_sim(golden, quirks=oracle.QUIRK_Q5_LHS if q5 else 0)
    set_fields(sim, golden["rand_cur"], ("curx", "cury", "curz"))
    sim.call("to_exchange_current")
    ref = golden["fold_q5" if q5 else "fold"]
    for a, n in zip(ref, ("curx", "cury", "curz")):
        np.testing.assert_array_equal(sim.fields[n], a, err_msg=n)


def test_filter(golden):
    sim = make_sim(golden)
    set_fields(sim, golden["fold"], ("curx", "cury", "curz"))
    sim.call("to_apply_filter1_opt")
    for a, n in zip(golden["filter2"], ("curx", "cury", "curz")):
        np.testing.assert_array_equal(sim.fields[n], a, err_msg=n)


def test_reorder(golden):
    sim = make_sim(golden)
    parts = golden["particles"].copy()
    mv = golden["moved"]
    for col, k in enumerate(("x", "y", "z", "u", "v", "w")):
        parts[k] = mv[:, col]
    sim.set_particles(parts, parts[:0])
    sim.call("to_reorder_particles_")
    np.testing.assert_array_equal(sim.ions, golden["reorder"])
