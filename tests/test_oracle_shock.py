"""Oracle restatement of the collisionless-shock pieces, pinned by known
answers: the Park-Miller minimal standard generator's published value
(seed 1, 10000 steps: 1043618065), correctly rounded sin/cos of single
arguments, Maxwell-Juttner tables and momenta with the right moments, the
injector's counts and ind sequence, and the wall (no particle is left
behind it, reflected particles move away from it)."""
import ctypes

import numpy as np
import pytest

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig


@pytest.fixture(scope="module")
def lib():
    oracle.build()
    return oracle.load()


def test_park_miller_known_answer(lib):
    d = ctypes.c_double(1.0)
    for _ in range(10000):
        lib.to_random(ctypes.byref(d))
    assert d.value == 1043618065.0


def test_random_is_seed_over_2_31_rounded_to_single(lib):
    d = ctypes.c_double(123457.0)
    for _ in range(1000):
        s_prev = d.value
        r = lib.to_random(ctypes.byref(d))
        assert d.value == (16807 * int(s_prev)) % 2147483647
        assert np.float32(r) == np.float32(d.value / 2147483648.0)


def test_sincos_correctly_rounded(lib):
    rng = np.random.default_rng(3)
    xs = (rng.random(20000) * 2 * np.pi).astype(np.float32)
    s, c = ctypes.c_float(), ctypes.c_float()
    for x in xs:
        lib.to_sincosf(float(x), ctypes.byref(s), ctypes.byref(c))
        assert np.float32(s.value) == np.float32(np.sin(np.float64(x)))
        assert np.float32(c.value) == np.float32(np.cos(np.float64(x)))


def test_maxwell_table_and_moments(lib):
    gt = (ctypes.c_float * oracle.PDF_SZ)()
    pt = (ctypes.c_float * (oracle.PDF_SZ + 1))()
    lib.to_init_maxw_table(1e-2, 2, 1.0, ctypes.addressof(gt), ctypes.addressof(pt))
    p = np.array(pt)
    assert p[0] == 0 and p[oracle.PDF_SZ - 1] == 1.0 and np.all(np.diff(p) >= 0)
    d = ctypes.c_double(987654.0)
    u, v, w = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
    us = []
    for _ in range(20000):
        lib.to_maxwell_dist(-15.0, 0.45, ctypes.byref(d), ctypes.byref(u), ctypes.byref(v), ctypes.byref(w),
                            ctypes.addressof(gt), ctypes.addressof(pt), 1.0, 1)
        us.append((u.value, v.value, w.value))
    us = np.array(us)
    # drifting Maxwell-Juttner: mean u = -gamma0 beta0 (1 + O(kT)), v, w symmetric
    g0 = 15.0
    assert us[:, 0].mean() == pytest.approx(-g0 * np.sqrt(1 - 1 / g0**2), rel=0.05)
    assert abs(us[:, 1].mean()) < 0.01 and abs(us[:, 2].mean()) < 0.01
    assert us[:, 1].std() == pytest.approx(np.sqrt(1e-2), rel=0.1)


def shock_sim(laps=0, fixed=1):
    cfg = SimConfig(dims=2, order=3, nx=96, ny=16, c=0.45, c_omp=4.0, ppc0=4.0, gamma0=15.0, delgam=1e-4,
                    sigma=0.1, ntimes=4, corr=1.0, periodic=(0, 1, 1), fixed=fixed)
    sh, f, reg = setups.shock_params(cfg)
    cfg.maxhlf = setups.shock_capacity(cfg, laps, sh)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.shock_init(sh)
    o.inject_region(*reg)
    return cfg, o, sh


def test_initial_load_counts_and_ind():
    cfg, o, sh = shock_sim()
    # numps = ceiling(0.5 ppc0 * 1 * 16 * (xinject2 - 20)) pairs
    n = int(np.ceil(np.float32(0.5 * 4.0) * np.float32(16.0) * np.float32(50.5 - 20.0)))
    assert o.st.ions == o.st.lecs == n
    np.testing.assert_array_equal(o.ions["ind"], 2 * np.arange(n) + 1)
    np.testing.assert_array_equal(o.lecs["ind"], 2 * np.arange(n) + 2)
    np.testing.assert_array_equal(o.ions["x"], o.lecs["x"])
    assert o.ions["x"].min() >= 20.0 and o.ions["x"].max() <= 50.5
    assert o.shock.totalpartnum == 2 * n


def test_wall_and_injector_over_laps():
    cfg, o, sh = shock_sim(laps=80)
    n0 = o.st.ions
    o.step_shock(80)
    per_lap = int(np.ceil(np.float32(2.0) * np.float32(16.0) * np.float32(np.float32(0.45) * np.float32(1.99999))))
    assert o.st.ions == o.st.lecs
    assert o.st.ions > n0 + 70 * (per_lap - 2) - 200  # injected minus the few removed at the boundaries
    assert o.shock.xinject2 == pytest.approx(50.5 + 80 * 0.45 * 0.99999, abs=1e-3)
    assert o.ions["x"].min() >= 20.0 and o.lecs["x"].min() >= 20.0
    refl = o.ions[o.ions["u"] > 0]
    assert len(refl) > 100 and refl["x"].min() >= 20.0
    # conductor behind the wall: ey = ez = 0 on columns 1..15
    ey = o.field("ey")[0]
    assert np.all(ey[:, :15] == 0)
