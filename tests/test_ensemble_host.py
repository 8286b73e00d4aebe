"""Host side of the batched ensemble: the seeded box table and the argument
checks of tg_ens_init (which run before any CUDA call)."""
import ctypes

import numpy as np
import pytest

from tristan_gb300 import setups


def test_ensemble_table_is_seeded_and_in_range():
    a, ta = setups.ensemble_configs(nbox=64, seed=3)
    b, tb = setups.ensemble_configs(nbox=64, seed=3)
    assert ta == tb
    assert len(a) == 64
    for c, t in zip(a, ta):
        assert c.dims == 2 and c.fixed == 1
        assert t["nx"] in setups.ENSEMBLE_SIDES and t["ny"] in setups.ENSEMBLE_SIDES
        assert 4 <= t["ppc_species"] <= 32 and t["ppc_species"] % 2 == 0
        assert 1.5 <= t["gamma0"] <= 10.0
        assert 1e-3 <= t["delgam"] <= 1e-1
        assert t["order"] in (1, 2, 3)
        assert c.ppc0 == 2 * t["ppc_species"] and c.order == t["order"]
    assert {t["order"] for t in ta} == {1, 2, 3}


def test_ensemble_loader_counts():
    cfgs, table = setups.ensemble_configs(nbox=3, seed=4, sides=(8, 12), ppc_range=(2, 6))
    parts = setups.load_ensemble(cfgs)
    for c, t, (ions, lecs) in zip(cfgs, table, parts):
        assert len(ions) == len(lecs) == c.nx * c.ny * t["ppc_species"]
        assert c.maxhlf >= len(ions)
        np.testing.assert_array_equal(ions["x"], lecs["x"])


def _init(cfgs):
    from tristan_gb300.gpu import load_library, make_tg_config, tg_config
    lib = load_library()
    arr = (tg_config * len(cfgs))(*[make_tg_config(c) for c in cfgs])
    h = ctypes.c_void_p()
    rc = lib.tg_ens_init(arr, len(cfgs), ctypes.byref(h))
    return rc, lib.tg_ens_last_error(None).decode()


@pytest.mark.parametrize("bad", ["dims", "periodic", "mode", "cadence"])
def test_ensemble_init_rejects_mixed_or_unsupported_boxes(bad):
    from tristan_gb300.gpu import TG_ERR_ARG
    cfgs, _ = setups.ensemble_configs(nbox=3, seed=5, sides=(16, 24))
    for c in cfgs:
        c.maxhlf = 4096
    if bad == "dims":
        cfgs[2].dims, cfgs[2].nz = 3, 16
    elif bad == "periodic":
        cfgs[1].periodic = (0, 1, 1)
    elif bad == "mode":
        cfgs[2].fixed = 0
    else:
        cfgs[1].sort_every = 3
    rc, msg = _init(cfgs)
    assert rc == TG_ERR_ARG
    assert "box" in msg
