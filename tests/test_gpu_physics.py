"""The physics known answers of the oracle tests, run through the CUDA
path itself (FP32 deposit, the mode the benchmark's value is quoted on):
plasma frequency, two-stream and Weibel growth rates, each against its
theory with the oracle's bars."""
import pytest

import physics_cases

pytestmark = pytest.mark.gpu


def gpu_runner(cfg, ions, lecs):
    from tristan_gb300.gpu import SYNC_B, SYNC_E, GpuSim
    cfg.fixed = 0
    g = gpu_runner.open = GpuSim(cfg)
    g.set_particles(ions, lecs)

    def step():
        g.step(1)
        g.sync_to_host(SYNC_E | SYNC_B)

    return step, g.field


@pytest.fixture(autouse=True)
def _close():
    gpu_runner.open = None
    yield
    if gpu_runner.open is not None:
        gpu_runner.open.close()


def test_gpu_plasma_oscillation_frequency():
    w, wp = physics_cases.plasma_oscillation(gpu_runner, 3)
    assert 0.998 < w / wp < 1.002, w / wp


def test_gpu_two_stream_growth_rate():
    rate, theory = physics_cases.two_stream(gpu_runner, 3)
    assert 0.95 < rate / theory < 1.03, (rate, theory)


@pytest.mark.parametrize("mode", [1, 3])
def test_gpu_weibel_growth_rate(mode):
    rate, theory = physics_cases.weibel(gpu_runner, 3, mode)
    assert 0.95 < rate / theory < 1.05, (rate, theory)
