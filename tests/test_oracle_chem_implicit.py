"""The oracle's restatement of the reference's time step with its complete model (ten species
and the potential; main.cpp:640-922): its eleven tangents equal utils::NewtonMatrices'
(utils.h:846-1849) bit for bit with the data files' constants and with constants that make
every linearised reaction term count; one step equals the reference's own functions
(Residuals, NewtonMatrices, Eigen::GMRES) assembled in main.cpp's loop; and a step converges,
keeps the Dirichlet values, the clamp and the flip rule.  Skipped where the reference's
sources are absent."""
import os

import numpy as np
import pytest

import chem_case
import chem_state

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "chemistry.npz")


def _case(nn, orc, kind, n, seed, reactive):
    g = np.load(GOLDEN)
    d2 = chem_case.reactive_data2(g["data2"]) if reactive else g["data2"].copy()
    dc, d11 = g["datac"], g["datac11"]
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(orc.synth, kind, n, seed, g["data2"])
    inp = orc.synth(kind, n, seed)
    p = nn.params_from_reference(d2, [dc[k] for k in range(4)], d11)
    o = orc.Oracle(p, nodes, inp["bctypes"], inp["bcvalues"], inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    bt, bv = chem_state.bc11(inp, Un, d2[7])
    return o, nodes, phase, Un, bt, bv, d2, dc, d11


@pytest.mark.parametrize("kind,n,seed", [(0, 12, 3), (1, 12, 3)])
@pytest.mark.parametrize("reactive", [False, True])
def test_chem_tangents_bit_exact_vs_reference(nn, orc, kind, n, seed, reactive):
    o, nodes, phase, U, bt, bv, d2, dc, d11 = _case(nn, orc, kind, n, seed, reactive)
    N = nodes.shape[1]
    lengths, ptr, cols = o.clouds()
    for f in range(11):
        ref = orc.ref_newton_k_full(f, nodes, ptr, cols, U, phase, bt, bv, chem_case.VOLN1REL, d2, dc, d11)
        if ref is None:
            pytest.skip("the reference's sources are not compiled here")
        diag, off = o.chem_tangent(f, U, phase, bt, bv, chem_case.VOLN1REL, d2, dc, d11)
        mine = {}
        for i in range(N):
            mine[(i, i)] = diag[i]
            for j in range(ptr[i] + 1, ptr[i + 1]):
                if off[j] != 0.0:
                    mine[(i, int(cols[j]))] = mine.get((i, int(cols[j])), 0.0) + off[j]
        theirs = {}
        for a, b, v in zip(*ref):
            theirs[(int(a), int(b))] = theirs.get((int(a), int(b)), 0.0) + v
        keys = set(mine) | set(theirs)
        bad = [k for k in keys if mine.get(k, 0.0) != theirs.get(k, 0.0)]
        assert not bad, (f, bad[:3])


def smooth_state(phase, d2):
    """A state near the model's own scales: uniform species in the liquid (1e-4 + 1e-5 k, in
    CSolid units), the solid's Mg at 1, a potential of zero."""
    N = phase.size
    U = np.zeros((11, N))
    for k in range(10):
        U[k] = 1e-4 + 1e-5 * k
    U[0][phase == 1] = 1.0
    return U


@pytest.mark.parametrize("kind,n,seed", [(1, 12, 5), (0, 14, 2)])
def test_chem_step_converges_and_keeps_the_rules(nn, orc, kind, n, seed):
    o, nodes, phase, _, bt, _, d2, dc, d11 = _case(nn, orc, kind, n, seed, False)
    inp = orc.synth(kind, n, seed)
    U = smooth_state(phase, d2)
    bt, bv = chem_state.bc11(inp, U, d2[7])
    U1, ph1, newton, krylov = o.chem_implicit_step(U, phase, bt, bv, chem_case.VOLN1REL, d2, dc, d11)
    assert 1 <= newton < 200 and krylov > 0
    assert np.isfinite(U1).all()
    cs = d2[7]
    for f in range(11):
        m = (bt == 0) & (bv[f] != -1)
        want = bv[f, m] / (cs if f < 10 else 1.0)
        assert np.allclose(U1[f, m], want, rtol=1e-9, atol=1e-14), f
    floor = 1e-8 / cs
    assert (U1[:9] >= floor).all()
    assert (U1[9][ph1 == 0] >= floor).all()
    # the flip rule (main.cpp:914-922): solid nodes at or below CSat/CSolid turn liquid
    csat = d2[8] / cs
    assert np.array_equal(ph1, np.where((phase == 1) & (U1[0] <= csat), 0, phase))
    assert np.abs(U1 - U).max() > 0.0


def _reference_step(orc, nodes, ptr, cols, U0, phase, bt, bv, voln1rel, d2, dc, d11):
    """main.cpp:640-922 assembled from the reference's own compiled functions (utils::Residuals,
    utils::NewtonMatrices and Eigen::GMRES through the shim), the loop's glue as written there:
    the Dirichlet rows (676-712), U += dU, the update norms, the clamp (805-837), the test
    max |res - res_old| < EPS (849-902) and the flip (914-922)."""
    N = nodes.shape[1]
    cs, csat = d2[7], d2[8] / d2[7]
    dirm = (bt[None, :] == 0) & (bv != -1)
    bcs = np.where(np.arange(11)[:, None] < 10, bv / cs, bv)
    U1 = U0.copy()
    res_old = np.zeros(11)
    newton = 0
    for it in range(200):
        F = orc.ref_residuals_full(nodes, ptr, cols, U1, U0, phase, voln1rel, d2, dc, d11)
        F = np.where(dirm, U1 - bcs, F)
        dU = np.empty_like(U1)
        for f in range(11):
            # the tangents of the step: NewtonMatrices at U^{n+1} = U^n (main.cpp:657)
            dU[f], _ = orc.ref_gmres_full(f, nodes, ptr, cols, U0, phase, bt, bv, voln1rel, d2, dc, d11, -F[f])
        U1 = U1 + dU
        res = np.sqrt((dU * dU).sum(axis=1))
        floor = 1.0e-8 / cs
        for k in range(10):
            m = U1[k] < floor
            if k == 9:
                m &= phase == 0
            U1[k][m] = floor
        newton = it + 1
        if np.abs(res - res_old).max() < 10e-6:
            break
        res_old = res
    ph = np.where((phase == 1) & (U1[0] <= csat), 0, phase).astype(np.int32)
    return U1, ph, newton


@pytest.mark.parametrize("perturbed", [False, True])
def test_chem_step_matches_the_reference_loop(nn, orc, perturbed):
    """One step of the oracle's restatement against the reference's own functions assembled
    in main.cpp's loop: the same Newton iteration count, the state to the GMRES tolerance's
    rounding, the same phases; from the smooth state and from it perturbed by 1% (every field
    moves, the potential too)."""
    if orc.load_reference() is None:
        pytest.skip("the reference's sources are not compiled here")
    o, nodes, phase, _, bt, _, d2, dc, d11 = _case(nn, orc, 1, 10, 5, False)
    inp = orc.synth(1, 10, 5)
    U = smooth_state(phase, d2)
    if perturbed:
        rng = np.random.default_rng(7)
        U = U * (1 + 0.01 * rng.standard_normal(U.shape))
        U[10] = 1e-3 * rng.standard_normal(U.shape[1])
    bt, bv = chem_state.bc11(inp, U, d2[7])
    lengths, ptr, cols = o.clouds()
    Ur, phr, nr = _reference_step(orc, nodes, ptr, cols, U, phase, bt, bv, chem_case.VOLN1REL, d2, dc, d11)
    Uo, pho, no, _ = o.chem_implicit_step(U, phase, bt, bv, chem_case.VOLN1REL, d2, dc, d11)
    assert no == nr
    assert np.array_equal(pho, phr)
    for f in range(11):
        scale = np.linalg.norm(Ur[f]) or 1.0
        assert np.linalg.norm(Uo[f] - Ur[f]) <= 1e-9 * scale, f


def test_four_species_step_matches_the_reference_loop(nn, orc):
    """The four-species implicit step (the handle's model, nnpp_forward_implicit's oracle) with
    the dissolution source off against the reference's own loop with reactions off and
    species 5-10 absent: fields 1-4 and the potential, the Newton count and the phases agree
    (within a step species 5-10 reach the others only through F11's charge of U^n, which is
    zero)."""
    if orc.load_reference() is None:
        pytest.skip("the reference's sources are not compiled here")
    g = np.load(GOLDEN)
    d2 = g["data2"].copy()
    d2[[29, 31, 33, 35, 37, 39, 41, 43, 45]] = 0.0
    d2[46] = 0.0
    dc, d11 = g["datac"], g["datac11"]
    p = nn.params_from_reference(d2, [dc[k] for k in range(4)], d11, k_diss=0.0)
    nodes, phase, _, _, r, cell = chem_case.case_inputs(orc.synth, 1, 10, 5, d2)
    inp = orc.synth(1, 10, 5)
    U = smooth_state(phase, d2)
    rng = np.random.default_rng(3)
    U[:4] *= 1 + 0.01 * rng.standard_normal((4, U.shape[1]))
    U[4:10] = 0.0
    U[10] = 1e-3 * rng.standard_normal(U.shape[1])
    bc5 = np.asarray(inp["bcvalues"], dtype=np.float64)
    o = orc.Oracle(p, nodes, inp["bctypes"], bc5, inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    o.set_state(U[:4], U[10], phase)
    v = o.diagnostics()["voln1rel"]
    lengths, ptr, cols = o.clouds()
    bt = np.asarray(inp["bctypes"], dtype=np.int32)
    bv = -np.ones((11, U.shape[1]))
    bv[:4] = bc5[:4]
    bv[10] = bc5[4]
    Ur, phr, nr = _reference_step(orc, nodes, ptr, cols, U, phase, bt, bv, v, d2, dc, d11)
    no, _ = o.implicit_forward(1)
    c, phi, ph, _ = o.state()
    assert no == nr
    assert np.array_equal(ph, phr)
    for k in range(4):
        assert np.linalg.norm(c[k] - Ur[k]) <= 1e-9 * np.linalg.norm(Ur[k]), k
    assert np.linalg.norm(phi - Ur[10]) <= 1e-9 * np.linalg.norm(Ur[10])
