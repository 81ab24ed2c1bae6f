"""The reference's implicit time step on the GPU (nnpp_forward_implicit; main.cpp:640-922)
against the oracle's restatement, which tests/test_oracle_implicit.py pins to the
reference's tangents and GMRES: the same Newton iteration counts, the states to the GMRES
tolerance's rounding, identical masks -- at the explicit step's dt and at ten times it (the
implicit step stays stable there), and with the explicit path continuing from the result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


def _pair(nn, orc, inp, p):
    sim = nn.Simulation(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    sim.build_neighbours()
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    return sim, o


@pytest.mark.parametrize("dt_scale", [1.0, 10.0])
def test_implicit_steps_match_oracle(gpu, orc, dt_scale):
    nn = gpu
    inp = nn.synth(1, 20, 9)
    p = inp["params"].copy()
    p.dt *= dt_scale
    sim, o = _pair(nn, orc, inp, p)
    for s in range(3):
        ng, kg = sim.forward_implicit(1)
        no, ko = o.implicit_forward(1)
        print("step %d dt x%g: newton gpu %d oracle %d, gmres gpu %d oracle %d" % (s, dt_scale, ng, no, kg, ko))
        assert ng == no
        assert abs(kg - ko) <= max(2, 0.02 * ko)
    c_g, phi_g, ph_g = sim.state()
    c_o, phi_o, ph_o, _ = o.state()
    ec = np.linalg.norm(c_g - c_o) / np.linalg.norm(c_o)
    ep = np.linalg.norm(phi_g - phi_o) / np.linalg.norm(phi_o)
    print("rel-L2 c %.2e phi %.2e" % (ec, ep))
    assert ec <= 1e-9 and ep <= 1e-9
    assert np.array_equal(ph_g, ph_o)
    assert sim.diagnostics()["steps_done"] == 3


def test_explicit_continues_after_implicit(gpu, orc):
    nn = gpu
    inp = nn.synth(1, 16, 4)
    sim, o = _pair(nn, orc, inp, inp["params"])
    sim.forward_implicit(2)
    o.implicit_forward(2)
    o.set_solver(1e-13)
    sim.set_solver(1e-12)
    sim.forward(20, nn.FP64)
    o.forward(20)
    c_g, phi_g, ph_g = sim.state()
    c_o, phi_o, ph_o, _ = o.state()
    assert np.linalg.norm(c_g - c_o) <= 1e-8 * np.linalg.norm(c_o)
    assert np.array_equal(ph_g, ph_o)
