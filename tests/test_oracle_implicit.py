"""The oracle's restatement of the reference's implicit time step (main.cpp:640-922), pinned
to the reference's own code compiled here (oracle/_ref): the tangents of
utils::NewtonMatrices (utils.h:844-1849) for the four species and the potential bit for bit,
and the Newton corrections' Eigen::GMRES solves (GMRES.h:56-203, as main.cpp:714-779 sets
them up) to rounding with the same iteration counts.  Skipped where the reference's sources
are absent."""
import os

import numpy as np
import pytest

CASES = [(1, 16, 3), (2, 12, 2)]


@pytest.fixture(scope="module")
def ref(orc):
    if orc.load_reference() is None:
        pytest.skip("reference sources not present")
    return orc


def _state(orc, kind, n, seed):
    inp = orc.synth(kind, n, seed)
    p = inp["params"].copy()
    p.k_diss = 0.0
    p.vol_red = 0.5
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    rng = np.random.default_rng(seed)
    N = inp["N"]
    c = 0.05 + rng.random((4, N))
    phi = rng.standard_normal(N) * 0.3
    ph = inp["phase0"].copy()
    o.set_state(c, phi, ph)
    return inp, p, o, c, phi, ph


@pytest.mark.parametrize("kind,n,seed", CASES)
def test_tangents_bit_exact_vs_reference(ref, kind, n, seed):
    orc = ref
    inp, p, o, c, phi, ph = _state(orc, kind, n, seed)
    N = inp["N"]
    lo, po, co = o.clouds()
    for f in range(5):
        diag, off = o.tangent(f)
        ri, ci, val = orc.ref_newton_k(f if f < 4 else 10, p, inp["nodes"], po, co, c, phi, ph,
                                       inp["bctypes"], inp["bcvalues"])
        mine = {}
        for i in range(N):
            mine[(i, i)] = diag[i]
            for j in range(po[i] + 1, po[i + 1]):
                if off[j] != 0.0:
                    mine[(i, int(co[j]))] = mine.get((i, int(co[j])), 0.0) + off[j]
        theirs = {}
        for r, q, v in zip(ri, ci, val):
            theirs[(int(r), int(q))] = theirs.get((int(r), int(q)), 0.0) + v
        keys = set(mine) | set(theirs)
        assert all(mine.get(k, 0.0) == theirs.get(k, 0.0) for k in keys), f


@pytest.mark.parametrize("kind,n,seed", CASES)
def test_gmres_matches_eigen(ref, kind, n, seed):
    orc = ref
    inp, p, o, c, phi, ph = _state(orc, kind, n, seed)
    lo, po, co = o.clouds()
    rng = np.random.default_rng(100 + seed)
    for f in range(5):
        b = rng.standard_normal(inp["N"])
        x, it = o.tangent_gmres(f, b)
        xr, itr = orc.ref_gmres(f if f < 4 else 10, p, inp["nodes"], po, co, c, phi, ph,
                                inp["bctypes"], inp["bcvalues"], b)
        assert it == itr, (f, it, itr)
        assert np.linalg.norm(x - xr) <= 1e-12 * np.linalg.norm(xr), f


def test_implicit_steps_converge(orc):
    inp = orc.synth(1, 14, 9)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    for _ in range(2):
        newton, krylov = o.implicit_forward(1)
        assert 1 <= newton < 200 and krylov > 0
    c, phi, ph, _ = o.state()
    assert np.isfinite(c).all() and np.isfinite(phi).all()


@pytest.mark.parametrize("kind,n,seed", [(0, 12, 3), (1, 12, 3)])
def test_implicit_residual_matches_reference(nn, orc, kind, n, seed):
    """The implicit step's residual (the time term, the bond sums at U^{n+1} with the migration
    in phi^n, F11 from phi^{n+1} and the charge of U^n) against the reference's own
    utils::Residuals on the same two time levels, with the reference's data files' constants
    and no reaction (rates and the H+ exchange current zero, k_diss = 0); species 5-10 absent."""
    import chem_case
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "chemistry.npz"))
    d2 = g["data2"].copy()
    d2[[29, 31, 33, 35, 37, 39, 41, 43, 45]] = 0.0  # k_b of the nine reactions
    d2[46] = 0.0                                    # JHp
    dc, d11 = g["datac"], g["datac11"]
    p = nn.params_from_reference(d2, [dc[k] for k in range(4)], d11, k_diss=0.0, switch_width=0.0)
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(orc.synth, kind, n, seed, d2)
    Un1[4:10] = 0.0
    Un[4:10] = 0.0
    inp = orc.synth(kind, n, seed)
    o = orc.Oracle(p, nodes, inp["bctypes"], inp["bcvalues"], inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    lengths, ptr, cols = o.clouds()
    Fr = orc.ref_residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    if Fr is None:
        pytest.skip("the reference's sources are not compiled here")
    F = o.residuals_implicit(Un1[:4], Un1[10], Un[:4], Un[10], phase, chem_case.VOLN1REL)
    for k, kr in ((0, 0), (1, 1), (2, 2), (3, 3), (4, 10)):
        scale = np.abs(Fr[kr]).max()
        assert np.abs(F[k] - Fr[kr]).max() <= 1e-12 * scale, k
    assert np.array_equal(F[4] == 0.0, Fr[10] == 0.0)
