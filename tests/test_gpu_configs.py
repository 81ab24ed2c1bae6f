"""Parity at the workloads' own sizes and lengths.

Each test runs one of the benchmark workloads at full size and states its error in the four
quantities every result reports (relative L2 of c and phi, front position in dx, Mg mass
lost), against the FP64 oracle where the oracle finishes in about a minute (it runs about
one second per step at 512,000 nodes on 16 host cores), and otherwise against the GPU's
FP64 path, which the other tests pin to the oracle:
  - jittered 80^3 lattice with a perturbed sphere (512,000 nodes): mixed and FP64 GPU runs
    against the oracle for 60 steps from t = 0; then 10,000 mixed steps against the FP64
    GPU path;
  - the permuted 2M-node screw: 500 mixed steps against the FP64 GPU path;
  - the calibration workload (262,144 nodes, 2,000 steps, checkpoints every 50): the mixed
    gradient (FP32 adjoint bond sums) against the FP64 GPU gradient, and the FP64 gradient
    against central differences (h = 1e-6 and 1e-4 relative) for D_0 and k;
  - an ensemble of uneven instances stepped in one batched launch: every member against
    its own oracle run.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

TOL_MIXED = 1e-5  # rel-L2 of c and phi, mixed precision against an FP64 run


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


def _sim(nn, inp, tol=1e-10):
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.set_solver(tol)
    return sim


def _errors(nn, p, run, ref):
    """run, ref: (c, phi, phase, mg_mass_lost)."""
    return nn.compare_states(p, run[0], run[1], run[2], ref[0], ref[1], ref[2], run[3], ref[3])


def _gpu_state(sim):
    c, phi, ph = sim.state()
    return c, phi, ph, sim.diagnostics()["mg_mass_lost"]


def _oracle_state(o):
    c, phi, ph, _ = o.state()
    return c, phi, ph, o.diagnostics()["mg_mass_lost"]


def test_sphere_512k_against_oracle(gpu, orc):
    """Jittered 80^3 lattice, perturbed sphere: 60 steps from t = 0, the mixed and the FP64
    GPU paths against the FP64 oracle (the same potential tolerance 1e-10 everywhere)."""
    nn = gpu
    inp = nn.synth(1, 80, 1)
    p = inp["params"]
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-10)
    o.forward(60)
    ref = _oracle_state(o)
    del o
    for prec, tol_c, tol_phi in ((nn.MIXED, TOL_MIXED, TOL_MIXED), (nn.FP64, 1e-9, 1e-8)):
        sim = _sim(nn, inp)
        sim.forward(60, prec)
        e = _errors(nn, p, _gpu_state(sim), ref)
        print("512k, 60 steps, %s vs oracle: %s" % ("mixed" if prec else "fp64", e))
        assert e["rel_l2_c"] <= tol_c and e["rel_l2_phi"] <= tol_phi, e
        assert e["mask_mismatch"] == 0 and e["front_dx"] == 0.0, e
        assert e["mg_mass_lost_rel"] <= 10 * tol_c, e


def test_sphere_512k_10000_steps_mixed_against_fp64(gpu):
    """The full 10,000 steps of the 512k workload: mixed against the FP64 GPU path (pinned to
    the oracle above and on the 8k lattice over 1,000 steps), compared every 2,000 steps."""
    nn = gpu
    inp = nn.synth(1, 80, 1)
    p = inp["params"]
    mixed, fp64 = _sim(nn, inp), _sim(nn, inp)
    solid0 = int(inp["phase0"].sum())
    for block in range(5):
        mixed.forward(2000, nn.MIXED)
        fp64.forward(2000, nn.FP64)
        e = _errors(nn, p, _gpu_state(mixed), _gpu_state(fp64))
        print("512k, %d steps, mixed vs fp64: %s" % (2000 * (block + 1), e))
        assert e["rel_l2_c"] <= TOL_MIXED and e["rel_l2_phi"] <= TOL_MIXED, e
        # a node within rounding of the saturation test may flip a step apart in the two
        # precisions; the front itself stays within a hundredth of a spacing
        assert e["front_dx"] <= 0.01, e
        assert e["mask_mismatch"] <= 1e-3 * max(solid0 - e["solid_nodes"], 1) + 2, e
        assert e["mg_mass_lost_rel"] <= TOL_MIXED, e
    assert e["solid_nodes"] < solid0  # the front moved


def test_screw_2m_500_steps_mixed_against_fp64(gpu):
    """The permuted 2M-node screw: 500 mixed steps against the FP64 GPU path."""
    nn = gpu
    inp = nn.synth(2, 126, 1)
    p = inp["params"]
    mixed, fp64 = _sim(nn, inp), _sim(nn, inp)
    mixed.forward(500, nn.MIXED)
    fp64.forward(500, nn.FP64)
    e = _errors(nn, p, _gpu_state(mixed), _gpu_state(fp64))
    print("2M screw, 500 steps, mixed vs fp64: %s" % e)
    assert e["rel_l2_c"] <= TOL_MIXED and e["rel_l2_phi"] <= TOL_MIXED, e
    assert e["mask_mismatch"] == 0 and e["mg_mass_lost_rel"] <= TOL_MIXED, e


def _calib_params(inp, scale_D=1.0, k=0.05):
    p = inp["params"].copy()
    p.switch_width = 0.01
    p.k_diss = k
    for s in range(4):
        p.D_liquid[s] *= scale_D
        p.D_solid[s] *= scale_D
    return p


def test_calibration_262k_2000_steps_gradients(gpu):
    """The calibration workload at its own size and length: jittered 64^3 lattice with an
    8-node Dirichlet shell, solid cylinder, loss = L2 misfit of the Mg mass-loss curve
    sampled every 20 steps against the curve at D x 1.2, k = 0.06; checkpoints every 50
    steps with recomputation.  The FP64 gradient agrees with central differences of the
    FP64 forward for D_0 and k, and the mixed gradient (FP32 adjoint bond sums) with the
    FP64 one.  Central differences at h = 1e-6 relative carry the potential solves' stopping
    noise (tolerance 1e-11, about 1e-5 of the gradient), so they are checked to 1e-3, and
    at h = 1e-4 (truncation ~1e-8) to 1e-5."""
    nn = gpu
    steps, ck, se = 2000, 50, 20
    inp = nn.synth(3, 64, 1)
    base = _calib_params(inp)
    sim = nn.Simulation(base, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"],
                        inp["phase0"])
    sim.build_neighbours()
    sim.set_solver(1e-11, 4000)
    sim.set_adjoint_store(1)  # checkpoints every ck steps, recomputation in backward
    sim.set_params(_calib_params(inp, 1.2, 0.06))
    target = sim.forward_ckpt(steps, nn.FP64, ck, se)
    sim.set_params(base)
    sim.reset()
    curve = sim.forward_ckpt(steps, nn.FP64, ck, se)
    gD, gk = sim.backward(2.0 * (curve - target))

    def loss(p):
        sim.set_params(p)
        sim.reset()
        c = sim.forward_ckpt(steps, nn.FP64, ck, se)
        return float(((c - target) ** 2).sum())

    def central(h):
        pp, pm = base.copy(), base.copy()
        for q, f in ((pp, 1 + h), (pm, 1 - h)):
            q.D_liquid[0] = base.D_liquid[0] * f
            q.D_solid[0] = base.D_solid[0] * f
        fd_D0 = (loss(pp) - loss(pm)) / (2 * h * base.D_liquid[0])
        pp, pm = base.copy(), base.copy()
        pp.k_diss = base.k_diss * (1 + h)
        pm.k_diss = base.k_diss * (1 - h)
        fd_k = (loss(pp) - loss(pm)) / (2 * h * base.k_diss)
        return fd_D0, fd_k

    for h, tol in ((1e-4, 1e-5), (1e-6, 1e-3)):
        fd_D0, fd_k = central(h)
        print("262k, 2000 steps, h=%g: grad D0 %.10e fd %.10e; grad k %.10e fd %.10e"
              % (h, gD[0], fd_D0, gk, fd_k))
        assert abs(gD[0] - fd_D0) <= tol * abs(fd_D0), (h, gD[0], fd_D0)
        assert abs(gk - fd_k) <= tol * abs(fd_k), (h, gk, fd_k)

    sim.set_params(base)
    sim.reset()
    sim.set_solver(1e-10, 4000)
    curve32 = sim.forward_ckpt(steps, nn.MIXED, ck, se)
    gD32, gk32 = sim.backward(2.0 * (curve32 - target))
    print("262k, 2000 steps: mixed grad D %s k %.10e; fp64 grad D %s k %.10e"
          % (list(gD32), gk32, list(gD), gk))
    assert np.abs(curve32 - curve).max() <= TOL_MIXED * np.abs(curve).max()
    assert abs(gD32[0] - gD[0]) <= 1e-4 * abs(gD[0]), (gD32, gD)
    assert abs(gk32 - gk) <= 1e-4 * abs(gk), (gk32, gk)
    assert np.linalg.norm(gD32 - gD) <= 1e-3 * np.linalg.norm(gD), (gD32, gD)


def test_ensemble_members_against_oracle(gpu, orc):
    """Four uneven ensemble members (own inclusion, diffusivities and rate) stepped together
    in one batched launch per step, each against its own FP64 oracle run."""
    nn = gpu
    inps = [nn.synth(4, n, 40 + i) for i, n in enumerate((24, 31, 27, 35))]
    sims = [_sim(nn, inp) for inp in inps]
    ens = nn.Ensemble(sims)
    ens.forward(100, nn.MIXED)
    for inp, sim in zip(inps, sims):
        o = orc.Oracle.from_synth(inp)
        o.build_neighbours()
        o.set_solver(1e-10)
        o.forward(100)
        e = _errors(nn, inp["params"], _gpu_state(sim), _oracle_state(o))
        print("ensemble member N=%d, 100 steps, mixed vs oracle: %s" % (inp["N"], e))
        assert e["rel_l2_c"] <= TOL_MIXED and e["rel_l2_phi"] <= TOL_MIXED, e
        assert e["mask_mismatch"] == 0 and e["mg_mass_lost_rel"] <= 10 * TOL_MIXED, e
    ens.close()
