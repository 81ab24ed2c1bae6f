"""Device-side checks and the bounded-wait failure path (nnpp_set_checks), without any GPU
fault: the checked build of the halo-staged CG operator gives the same bits as the plain one
on valid inputs, and a wait that is made to run out (on a barrier that nothing completes,
after every copy has landed) comes back as NNPP_ERR_CUDA, after which the same handle runs
normally again."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HALO_OPERATOR = 8


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


def _sim(nn, inp):
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.set_tuning(4, 8, HALO_OPERATOR)
    return sim


def test_bounds_checks_change_nothing(gpu):
    nn = gpu
    inp = nn.synth(1, 20, seed=5)
    plain, checked = _sim(nn, inp), _sim(nn, inp)
    checked.set_checks(nn.CHECK_BOUNDS)
    plain.forward(60, nn.MIXED)
    checked.forward(60, nn.MIXED)
    for a, b in zip(plain.state(), checked.state()):
        assert np.array_equal(a, b)


def test_wait_probe_reports_timeout_and_handle_recovers(gpu):
    nn = gpu
    inp = nn.synth(1, 20, seed=5)
    ref = _sim(nn, inp)
    ref.forward(20, nn.MIXED)
    sim = _sim(nn, inp)
    sim.set_solver(1e-10, 30)
    sim.set_checks(nn.CHECK_WAIT_PROBE)
    with pytest.raises(nn.NNPPError) as e:
        sim.forward(1, nn.MIXED)
    assert e.value.status == 5  # NNPP_ERR_CUDA
    assert "timed out" in str(e.value)
    sim.set_checks(0)
    sim.set_solver(1e-10, 2000)
    sim.reset()
    sim.forward(20, nn.MIXED)
    for a, b in zip(ref.state(), sim.state()):
        assert np.array_equal(a, b)


def test_set_checks_rejects_unknown_flags(gpu):
    nn = gpu
    sim = nn.Simulation.from_synth(nn.synth(1, 12, seed=4))
    with pytest.raises(nn.NNPPError) as e:
        sim.set_checks(4)
    assert e.value.status == 1
