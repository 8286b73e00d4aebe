"""Output moments (meanq_fld_cur, code/output.F90:5222-5482) on the device
against the oracle's restatement: number densities of unit-weight
particles are sums of integers, hence bit-exact; the velocity, momentum and
energy moments (FP64 sums on the device, sequential single-precision sums
in the reference) agree to 1e-5 norm-wise and 1e-4 of the maximum per
element."""
import numpy as np
import pytest

import oracle
from test_gpu_parity import beams, random_fields, small_cfg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,order", [(2, 3), (3, 2)])
def test_moments_match_oracle(dims, order):
    from tristan_gb300.gpu import GpuSim, MOMENTS
    cfg = small_cfg(dims, order, fixed=1)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(3), scale=0.02)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs)
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.set_particles(ions, lecs)
    g.step(2)
    o.step(2)
    cur_before = o.fields["curx"].copy()
    for kind, name in enumerate(MOMENTS):
        gn, gd = g.meanq(name)
        on, od = o.meanq(kind)
        if name in ("tdens", "idens"):
            np.testing.assert_array_equal(gn, on, err_msg=name)
        else:
            for got, ref in ((gn, on), (gd, od)):
                nrm = max(np.linalg.norm(ref.astype(np.float64)), 1e-30)
                assert np.linalg.norm(got.astype(np.float64) - ref) / nrm <= 1e-5, name
                assert np.abs(got - ref).max() <= 1e-4 * max(np.abs(ref).max(), 1e-30), name
    np.testing.assert_array_equal(o.fields["curx"], cur_before)  # the oracle restores the currents
    # the device run continues unaffected by the moments' scratch use
    g.step(1)
    o.step(1)
    g.sync_to_host()
    for k in ("ex", "ey", "ez", "bx", "by", "bz"):
        np.testing.assert_array_equal(g.fields[k], o.fields[k], err_msg=k)
    g.close()


def test_flow_frame_spectra_match_oracle():
    """save_spectrum_2d on the device: slice and gamma axes and the gamma
    range equal the oracle's; the histograms agree except for particles
    whose flow-frame gamma sits on a bin edge (the slice means are summed in
    a different order): at most a few per mille of the weight moves. The
    plasma is warm (kT = 0.01, gamma0 = 3): for a cold relativistic beam
    gamma' - 1 is a difference of nearly equal single-precision numbers, so
    any change of the summation order of the slice means moves most
    particles between bins, in the reference as well."""
    from tristan_gb300.gpu import GpuSim
    cfg = small_cfg(2, 3, fixed=1, nx=64, ny=40, ppc0=16.0)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(4), scale=0.02)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs)
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.set_particles(ions, lecs)
    g.step(5)
    o.step(5)
    gs = g.spectrum()
    os_ = o.spectrum()
    for k in ("xgamma", "xslice", "yslice"):
        np.testing.assert_array_equal(gs[k], os_[k], err_msg=k)
    assert gs["gammin"] == os_["gammin"] and gs["gammax"] == os_["gammax"]
    for sp in ("ions", "lecs"):
        a, b = gs[sp].astype(np.float64), os_[sp].astype(np.float64)
        tot = b.sum()
        assert tot > 10000
        assert abs(a.sum() - tot) <= 2
        assert np.abs(a - b).sum() <= max(4.0, 2e-3 * tot), sp
    g.close()


def test_x_slice_spectra_match_oracle():
    """save_spectrum (the writer the reference's output calls) on the device:
    x slices of about 100 cells, lab-frame and flow-frame spectra with the
    splitratio^(1 - splitlev) weights, divided by gamma - 1. Axes and the
    gamma range equal the oracle's; lab-frame bins are the same per
    particle, so the sums agree to FP32 summation order; flow-frame bins
    move by a few per mille of the weight at most, as for the 2D writer"""
    from tristan_gb300.gpu import GpuSim
    cfg = small_cfg(2, 3, fixed=1, nx=320, ny=16, ppc0=8.0)
    ions, lecs = beams(cfg)
    ions["splitlev"][::7] = 2   # weight 0.1
    lecs["splitlev"][::5] = 3   # weight 0.01
    f = random_fields(cfg, np.random.default_rng(5), scale=0.02)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs)
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.set_particles(ions, lecs)
    g.step(5)
    o.step(5)
    gs = g.spectrum_x()
    os_ = o.spectrum_x()
    assert gs["xslice"].size == 3
    for k in ("xgamma", "xslice"):
        np.testing.assert_array_equal(gs[k], os_[k], err_msg=k)
    assert gs["gammin"] == os_["gammin"] and gs["gammax"] == os_["gammax"]
    xg = gs["xgamma"].astype(np.float64)[:, None]
    for sp in ("ions", "lecs"):
        lab_g, lab_o = gs[sp] * xg, os_[sp] * xg
        tot = lab_o.sum()
        assert tot > 1000
        np.testing.assert_allclose(lab_g, lab_o, rtol=1e-5, atol=1e-6 * tot, err_msg=sp)
        rest_g, rest_o = gs[sp + "_rest"] * xg, os_[sp + "_rest"] * xg
        assert abs(rest_g.sum() - rest_o.sum()) <= 1e-5 * tot + 2
        assert np.abs(rest_g - rest_o).sum() <= max(4.0, 2e-3 * tot), sp
    g.close()


@pytest.mark.parametrize("dims,order,ext", [(2, 3, False), (2, 1, True), (3, 2, False)])
def test_output_tot_matches_oracle(dims, order, ext):
    """output_tot's variables sampled on the device: E and B through
    interpolfld (plus the constant external field), the currents and the
    moments, at istep 2 and 3 (the sampled range then starts and ends
    inside the array). Fields and currents bit-exact, densities exact,
    velocity moments within 1e-5"""
    from tristan_gb300.gpu import MOMENTS, GpuSim
    kw = dict(external_fields=1, ext=(0.0, 0.0, 0.0, 0.0, 0.0, 0.05)) if ext else {}
    cfg = small_cfg(dims, order, fixed=1, **kw)
    ions, lecs = beams(cfg)
    f = random_fields(cfg, np.random.default_rng(6), scale=0.02)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs)
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.set_particles(ions, lecs)
    g.step(3)
    o.step(3)
    for istep in (2, 3):
        for name, code in GpuSim.OUTPUT_VARS.items():
            a, b = g.output_var(name, istep), o.output_var(code, istep)
            assert a.shape == b.shape and a.size > 0
            np.testing.assert_array_equal(a, b, err_msg=f"{name} istep {istep}")
        for name in ("tdens", "idens"):
            np.testing.assert_array_equal(g.output_var(name, istep), o.output_var(16 + MOMENTS.index(name), istep),
                                          err_msg=name)
        for name in ("tbetx", "imomy", "iener"):
            a, b = g.output_var(name, istep), o.output_var(16 + MOMENTS.index(name), istep)
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6 * max(np.abs(b).max(), 1e-30), err_msg=name)
    g.close()


@pytest.mark.parametrize("dims,order", [(2, 3), (3, 2)])
def test_output_particle_sample_matches_oracle(dims, order):
    """output_tot's particle sample (prtl.tot) on the device: the same
    particles (modulo(ind / 2, stride) = 0, compared keyed by ind) with the
    same values bit for bit; negative ind (beam particles) included"""
    from tristan_gb300.gpu import GpuSim
    cfg = small_cfg(dims, order, fixed=1)
    ions, lecs = beams(cfg)
    ions["ind"][::5] *= -1
    f = random_fields(cfg, np.random.default_rng(8), scale=0.02)
    o = oracle.OracleSim(cfg)
    for k, v in f.items():
        o.fields[k][:] = v
    o.set_particles(ions, lecs)
    g = GpuSim(cfg)
    g.set_fields(**f)
    g.sync_from_host()
    g.set_particles(ions, lecs)
    g.step(3)
    o.step(3)
    for species in (0, 1):
        for stride in (1, 3, 10):
            a, b = g.output_particles(species, stride), o.output_particles(species, stride)
            assert len(a["ind"]) == len(b["ind"]) > 0
            ia, ib = np.argsort(a["ind"], kind="stable"), np.argsort(b["ind"], kind="stable")
            for k in a:
                np.testing.assert_array_equal(a[k][ia], b[k][ib], err_msg=f"{species} {stride} {k}")
    g.close()
