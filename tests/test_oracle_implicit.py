"""The oracle's restatement of the reference's implicit time step (main.cpp:640-922), pinned
to the reference's own code compiled here (oracle/_ref): the tangents of
utils::NewtonMatrices (utils.h:844-1849) for the four species and the potential bit for bit,
and the Newton corrections' Eigen::GMRES solves (GMRES.h:56-203, as main.cpp:714-779 sets
them up) to rounding with the same iteration counts.  Skipped where the reference's sources
are absent."""
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
