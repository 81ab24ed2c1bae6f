"""GPU checkpointed adjoint (nnpp_forward_ckpt / nnpp_backward) against the oracle's FP64
adjoint, against central finite differences of the GPU forward, across checkpoint intervals
and precisions, and through the torch.autograd binding."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_STEPS, SE = 60, 20


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


def _params(inp, scale_D=1.0, k=0.05):
    p = inp["params"].copy()
    p.switch_width = 0.01
    p.k_diss = k
    for s in range(4):
        p.D_liquid[s] *= scale_D
        p.D_solid[s] *= scale_D
    return p


@pytest.fixture(scope="module")
def case(gpu, orc):
    inp = gpu.synth(1, 12, 5)
    o = orc.Oracle(_params(inp, 1.2, 0.06), inp["nodes"], inp["bctypes"], inp["bcvalues"],
                   inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    o.set_solver(1e-14)
    target = orc.oracle_forward_record(o, N_STEPS, SE)
    return inp, target


def _sim(nn, inp, p, tol=1e-13, pin=False):
    """pin: a fixed execution configuration (the autotuner's timing-based choice changes the
    summation order, so bit-for-bit comparisons between handles pin it)."""
    sim = nn.Simulation(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"],
                        inp["phase0"])
    sim.build_neighbours()
    sim.set_solver(tol, 4000)
    if pin:
        sim.set_tuning(4, 8, 0)
    return sim


def test_adjoint_fp64_matches_oracle(gpu, orc, case):
    inp, target = case
    p = _params(inp)
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    o.set_solver(1e-14)
    curve_o = orc.oracle_forward_record(o, N_STEPS, SE)
    gD_o, gk_o = orc.oracle_backward(o, 2.0 * (curve_o - target))
    sim = _sim(gpu, inp, p)
    curve = sim.forward_ckpt(N_STEPS, gpu.FP64, 25, SE)
    np.testing.assert_allclose(curve, curve_o, rtol=1e-10)
    gD, gk = sim.backward(2.0 * (curve - target))
    # species 0 and the rate constant to 1e-8; species 1-3 act through the potential only
    # (gradients 100-1000x smaller) and carry the solves' 1e-13 tolerance
    assert abs(gD[0] - gD_o[0]) <= 1e-8 * abs(gD_o[0]), (gD, gD_o)
    for k in range(1, 4):
        assert abs(gD[k] - gD_o[k]) <= 1e-5 * abs(gD_o[k]), (k, gD, gD_o)
    assert abs(gk - gk_o) <= 1e-8 * abs(gk_o), (gk, gk_o)


def test_adjoint_fp64_matches_central_differences(gpu, case):
    inp, target = case
    base = _params(inp)
    sim = _sim(gpu, inp, base)
    curve = sim.forward_ckpt(N_STEPS, gpu.FP64, 25, SE)
    gD, gk = sim.backward(2.0 * (curve - target))

    def loss(p):
        sim.set_params(p)
        sim.reset()
        c = sim.forward_ckpt(N_STEPS, gpu.FP64, 25, SE)
        return float(((c - target) ** 2).sum())

    h = 1e-5
    tol = (1e-7, 1e-4, 1e-4, 1e-4)
    for k in range(4):
        pp, pm = base.copy(), base.copy()
        v = base.D_liquid[k]
        for q, f in ((pp, 1 + h), (pm, 1 - h)):
            q.D_liquid[k] = v * f
            q.D_solid[k] = base.D_solid[k] * f
        fd = (loss(pp) - loss(pm)) / (2 * h * v)
        assert abs(gD[k] - fd) <= tol[k] * abs(fd), (k, gD[k], fd)
    pp, pm = base.copy(), base.copy()
    pp.k_diss = base.k_diss * (1 + h)
    pm.k_diss = base.k_diss * (1 - h)
    fd = (loss(pp) - loss(pm)) / (2 * h * base.k_diss)
    assert abs(gk - fd) <= 1e-8 * abs(fd), (gk, fd)


def test_checkpoint_interval_does_not_change_result(gpu, case):
    """Segments are recomputed from checkpoints by the same deterministic kernels, so the
    gradients do not depend on the checkpoint interval."""
    inp, target = case
    out = []
    for ck in (7, 25, 60):
        sim = _sim(gpu, inp, _params(inp), pin=True)
        sim.set_adjoint_store(1)
        curve = sim.forward_ckpt(N_STEPS, gpu.FP64, ck, SE)
        gD, gk = sim.backward(2.0 * (curve - target))
        out.append((curve, gD, gk))
    for curve, gD, gk in out[1:]:
        assert np.array_equal(curve, out[0][0])
        assert np.array_equal(gD, out[0][1])
        assert gk == out[0][2]


@pytest.mark.parametrize("store", [1, 3])
def test_checkpoint_invariance_with_coarse_rebuilds(gpu, case, store):
    """The implant dissolves between steps 35 and 40 (k_diss = 0.1), so the coarse operator of
    the two-level preconditioner is rebuilt during the forward run (refresh period 4);
    backward replays the recorded inverses (for the adjoint solves, and with store 3 for the
    recomputed forward solves too), and the gradients stay independent of the checkpoint
    interval, and equal to a run that never rebuilds to the solver tolerance."""
    inp, _ = case
    p = _params(inp, 1.0, 0.1)
    target = np.zeros(N_STEPS // SE)
    out = []
    for every, ck in ((4, 7), (4, 25), (4, 60), (0, 25)):
        sim = _sim(gpu, inp, p, pin=True)
        sim.set_adjoint_store(store)
        sim.set_preconditioner(gpu.PRECOND_TWO_LEVEL, every)
        curve = sim.forward_ckpt(N_STEPS, gpu.FP64, ck, SE)
        built = sim.preconditioner()[3]
        assert built >= 2 if every else built == 1
        gD, gk = sim.backward(2.0 * (curve - target))
        assert sim.preconditioner()[3] == built
        out.append((curve, gD, gk))
    for curve, gD, gk in out[1:3]:
        assert np.array_equal(curve, out[0][0])
        assert np.array_equal(gD, out[0][1])
        assert gk == out[0][2]
    curve, gD, gk = out[3]
    assert np.allclose(curve, out[0][0], rtol=1e-9, atol=0)
    assert np.allclose(gD, out[0][1], rtol=1e-6, atol=1e-12 * np.abs(out[0][1]).max())
    assert abs(gk - out[0][2]) <= 1e-6 * abs(out[0][2])


@pytest.mark.parametrize("prec", [0, 1])
def test_stored_snapshots_equal_recomputation(gpu, case, prec):
    """Keeping every step's snapshot (no recomputation), recomputing checkpoint segments from
    the stored potentials (bond sums only) and recomputing them whole give the same curve and
    gradients bit for bit, and the automatic mode picks one of them."""
    inp, target = case
    out = []
    for mode in (1, 2, 3, 0):
        sim = _sim(gpu, inp, _params(inp), pin=True)
        sim.set_adjoint_store(mode)
        curve = sim.forward_ckpt(N_STEPS, prec, 25, SE)
        gD, gk = sim.backward(2.0 * (curve - target))
        out.append((curve, gD, gk, sim.state()))
    for curve, gD, gk, state in out[1:]:
        assert np.array_equal(curve, out[0][0])
        assert np.array_equal(gD, out[0][1])
        assert gk == out[0][2]
        for a, b in zip(state, out[0][3]):
            assert np.array_equal(a, b)


def test_adjoint_store_rejects_bad_mode(gpu, case):
    inp, _ = case
    sim = _sim(gpu, inp, _params(inp))
    for bad in (-1, 4):
        with pytest.raises(gpu.NNPPError) as e:
            sim.set_adjoint_store(bad)
        assert e.value.status == 1


def test_backward_restores_end_state(gpu, case):
    inp, target = case
    sim = _sim(gpu, inp, _params(inp))
    curve = sim.forward_ckpt(N_STEPS, gpu.FP64, 25, SE)
    c0, phi0, ph0 = sim.state()
    sim.backward(2.0 * (curve - target))
    c1, phi1, ph1 = sim.state()
    assert np.array_equal(c0, c1) and np.array_equal(phi0, phi1) and np.array_equal(ph0, ph1)


def test_adjoint_mixed_close_to_fp64(gpu, case):
    inp, target = case
    g = {}
    for prec in (gpu.FP64, gpu.MIXED):
        sim = _sim(gpu, inp, _params(inp), tol=1e-12)
        curve = sim.forward_ckpt(N_STEPS, prec, 25, SE)
        g[prec] = sim.backward(2.0 * (curve - target))
    (gD64, gk64), (gD32, gk32) = g[gpu.FP64], g[gpu.MIXED]
    assert abs(gD32[0] - gD64[0]) <= 1e-5 * abs(gD64[0])
    assert abs(gk32 - gk64) <= 1e-5 * abs(gk64)
    assert np.linalg.norm(gD32 - gD64) <= 1e-3 * np.linalg.norm(gD64)


def test_adjoint_solver_tolerance_and_stats(gpu, case):
    """The mixed adjoint's potential solves run to 1e-8 by default: the gradient moves by far
    less than the mixed-vs-FP64 difference when they run to 1e-12 instead, at more inner
    iterations; the per-step iteration log adds up to the reported total, one solve a step."""
    inp, target = case
    res = {}
    for tol in (0.0, 1e-12):
        sim = _sim(gpu, inp, _params(inp), tol=1e-12, pin=True)
        sim.set_adjoint_solver(tol)
        curve = sim.forward_ckpt(N_STEPS, gpu.MIXED, 25, SE)
        gD, gk = sim.backward(2.0 * (curve - target))
        res[tol] = (gD, gk, sim.adjoint_stats(per_step=True))
    (gD0, gk0, st0), (gD1, gk1, st1) = res[0.0], res[1e-12]
    assert np.linalg.norm(gD0 - gD1) <= 1e-7 * np.linalg.norm(gD1)
    assert abs(gk0 - gk1) <= 1e-7 * abs(gk1)
    for st in (st0, st1):
        assert st["solves"] == N_STEPS
        assert st["sweeps"] >= st["solves"]
        assert st["per_step"].shape == (N_STEPS,)
        assert int(st["per_step"].sum()) == st["cg_iterations"]
        assert (st["per_step"] >= 0).all() and st["cg_iterations"] > 0
    assert st1["cg_iterations"] > st0["cg_iterations"]
    sim = _sim(gpu, inp, _params(inp))
    for bad in (-1.0, 1.0, float("nan")):
        with pytest.raises(gpu.NNPPError) as e:
            sim.set_adjoint_solver(bad)
        assert e.value.status == 1


def test_backward_errors(gpu, case):
    inp, _ = case
    sim = _sim(gpu, inp, _params(inp))
    with pytest.raises(gpu.NNPPError) as e:
        sim.backward(np.zeros(3))
    assert e.value.status == 7  # NNPP_ERR_STATE: no recorded forward
    sim.forward_ckpt(N_STEPS, gpu.FP64, 25, SE)
    p = _params(inp)
    p.delta *= 1.01
    with pytest.raises(gpu.NNPPError) as e:
        sim.set_params(p)
    assert e.value.status == 1


def test_torch_autograd_binding(gpu, orc, case):
    torch = pytest.importorskip("torch")
    ag = importlib.import_module("nnpp_gb300.autograd")
    inp, target = case
    base = _params(inp)
    sim = _sim(gpu, inp, base)
    theta = torch.tensor(list(base.D_liquid) + [base.k_diss], dtype=torch.float64,
                         requires_grad=True)
    curve = ag.mass_loss_curve(theta, sim, base, N_STEPS, gpu.FP64, 25, SE)
    loss = ((curve - torch.from_numpy(target)) ** 2).sum()
    loss.backward()
    o = orc.Oracle(base, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    o.set_solver(1e-14)
    curve_o = orc.oracle_forward_record(o, N_STEPS, SE)
    gD_o, gk_o = orc.oracle_backward(o, 2.0 * (curve_o - target))
    ref = np.concatenate([gD_o, [gk_o]])
    got = theta.grad.numpy()
    assert abs(got[0] - ref[0]) <= 1e-8 * abs(ref[0])
    assert abs(got[4] - ref[4]) <= 1e-8 * abs(ref[4])
    # species 1-3 act through the potential only (gradients 100-1000x smaller) and carry the
    # solves' tolerance, as in test_adjoint_fp64_matches_oracle
    for k in range(1, 4):
        assert abs(got[k] - ref[k]) <= 1e-5 * abs(ref[k]), (k, got, ref)
    # a second call from the reset state gives the same curve
    curve2 = ag.mass_loss_curve(theta.detach(), sim, base, N_STEPS, gpu.FP64, 25, SE)
    assert torch.equal(curve.detach(), curve2)
