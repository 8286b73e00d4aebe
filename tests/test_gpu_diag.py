"""FP64 diagnostics on the device against the FP64 CPU oracle.

The device computes each particle's charge weights in FP32 and sums them in
int64 fixed point, gamma-1 as u^2/(gamma+1) in FP32 and all sums in FP64;
the oracle does every product in FP64. Stated error bound: 1e-6 relative
(momenta: 1e-6 of the summed |m u| scale); the Gauss residual itself is
checked in units of |F(rho)|.
"""
import numpy as np
import pytest

import oracle
from tristan_gb300 import setups
from tristan_gb300.config import SimConfig

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,order", [(2, 1), (2, 3), (3, 2)])
def test_diagnostics_match_oracle(dims, order):
    from tristan_gb300.gpu import GpuSim
    if dims == 2:
        cfg = SimConfig(dims=2, order=order, nx=48, ny=32, c_omp=4.0, ppc0=8.0, gamma0=3.0, ntimes=4,
                        fixed=1, diag_every=1)
    else:
        cfg = SimConfig(dims=3, order=order, nx=12, ny=12, nz=12, c_omp=4.0, ppc0=4.0, gamma0=3.0, ntimes=2,
                        fixed=1, diag_every=1)
    ions, lecs = setups.load_beams(cfg, seed=5)
    setups.with_capacity(cfg, len(ions), len(lecs))
    o = oracle.OracleSim(cfg)
    o.set_particles(ions, lecs)
    g = GpuSim(cfg)
    g.set_particles(ions, lecs)
    g.step(6)
    o.step(6)
    ref = o.diagnostics()
    got = g.diagnostics()
    hist = g.diag_history(6)
    assert hist.shape == (6, 16)
    g.close()
    rn = ref["rho_norm"]
    assert rn > 0
    assert abs(got["rho_norm"] - rn) <= 1e-6 * rn
    assert abs(got["gauss_abs"] - ref["gauss_abs"]) <= 1e-6 * rn
    # the residual is the reference arithmetic's own rounding floor: the
    # device's value tracks the oracle's (charge weights in FP32 there, FP64
    # here), and against one species' charge density it is below 1e-5
    assert abs(got["gauss_residual"] - ref["gauss_residual"]) <= 0.02 * ref["gauss_residual"]
    ncell = cfg.interior_cells
    norm_s = (abs(cfg.qi) * len(ions) + abs(cfg.qe) * len(lecs)) / (2.0 * ncell) * np.sqrt(ncell)
    assert got["gauss_abs"] / norm_s <= 1e-5
    for k in ("e_field", "e_mag", "e_kin_ions", "e_kin_lecs"):
        assert abs(got[k] - ref[k]) <= 1e-6 * max(abs(ref[k]), 1e-30), k
    scale = ref["e_kin_ions"] + ref["e_kin_lecs"]
    for a in range(3):
        assert abs(got["p_part"][a] - ref["p_part"][a]) <= 1e-6 * scale
        assert abs(got["p_field"][a] - ref["p_field"][a]) <= 1e-6 * max(abs(ref["e_field"]), 1e-30) * 10
    # the in-graph history's last record is the same state's diagnostics
    last = hist[-1]
    assert abs(np.sqrt(last[1]) - got["rho_norm"]) <= 1e-12 * rn
