"""The oracle (FP64 CPU restatement) against the reference: committed golden fixtures made
from the reference's own grid.h/utils.h (tests/golden/make_golden.py), and, where the
reference's sources are present, the reference itself, bit for bit."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR


def _golden(name):
    with open(os.path.join(GOLDEN_DIR, name)) as f:
        return json.load(f)


def _digest(lengths, cols):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(lengths, dtype=np.int32).tobytes())
    h.update(np.ascontiguousarray(cols, dtype=np.int32).tobytes())
    return h.hexdigest()


SMALL = [(0, 20, 11), (1, 16, 11), (2, 14, 11), (3, 20, 11), (4, 15, 11)]


@pytest.mark.parametrize("kind,n,seed", SMALL)
def test_oracle_clouds_match_reference_golden(nn, orc, kind, n, seed):
    g = _golden("clouds.json")["kind%d_n%d_seed%d" % (kind, n, seed)]
    inp = nn.synth(kind, n, seed)
    o = orc.Oracle.from_synth(inp)
    ml = o.build_neighbours()
    lo, po, co = o.clouds()
    assert ml == g["max_len"] and int(po[-1]) == g["nnz"]
    assert _digest(lo, co) == g["sha256"]


def test_oracle_clouds_lattice_block_8k_golden(nn, orc):
    g = _golden("clouds.json")["lattice_block_20"]
    inp = nn.synth(g["kind"], g["n_side"], g["seed"])
    o = orc.Oracle.from_synth(inp)
    assert o.build_neighbours() == g["max_len"]
    lo, po, co = o.clouds()
    assert _digest(lo, co) == g["sha256"]


@pytest.mark.slow
def test_oracle_clouds_512k_golden(nn, orc):
    g = _golden("clouds.json")["jittered_sphere_80"]
    inp = nn.synth(g["kind"], g["n_side"], g["seed"])
    o = orc.Oracle.from_synth(inp)
    assert o.build_neighbours() == g["max_len"]
    lo, po, co = o.clouds()
    assert int(po[-1]) == g["nnz"] and _digest(lo, co) == g["sha256"]


def test_synth_inputs_are_the_fixtures_inputs(nn):
    """The generator reproduces the coordinates the fixtures were made from (bit for bit,
    on any host: only IEEE +,-,*,/,sqrt, no FMA contraction)."""
    g = _golden("synth.json")
    for kind, n, seed in SMALL:
        inp = nn.synth(kind, n, seed)
        h = hashlib.sha256(np.ascontiguousarray(inp["nodes"]).tobytes()).hexdigest()
        assert h == g["kind%d_n%d_seed%d" % (kind, n, seed)]


@pytest.mark.parametrize("kind,n,seed", [(0, 12, 3), (1, 12, 3), (2, 12, 3)])
def test_oracle_residuals_match_reference_golden(nn, orc, kind, n, seed):
    F_ref = np.load(os.path.join(GOLDEN_DIR, "residuals.npz"))["kind%d_n%d_seed%d_F" % (kind, n, seed)]
    inp = nn.synth(kind, n, seed)
    p = inp["params"].copy()
    p.k_diss = 0.0
    p.vol_red = 0.5
    N = inp["N"]
    rng = np.random.default_rng(100 + kind)
    c = 0.05 + rng.random((4, N))
    phi = rng.standard_normal(N) * 0.3
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    F = o.residuals(c, phi, inp["phase0"], voln1rel=0.25)
    assert np.array_equal(F, F_ref)  # bit for bit


def test_oracle_k11_matches_reference_golden(nn, orc):
    g = _golden("k11.json")
    inp = nn.synth(1, 12, 3)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    lo, po, co = o.clouds()
    diag, off, free = o.poisson_matrix(inp["phase0"])
    N = inp["N"]
    rows = np.repeat(np.arange(N), np.diff(po)).astype(np.int64)
    ent = {}
    for r, cc, v in zip(rows, co, off):
        if r != cc and v != 0.0:
            ent[(int(r), int(cc))] = v
    for i in range(N):
        ent[(i, i)] = diag[i]
    keys = sorted(ent)
    ri = np.array([k[0] for k in keys], dtype=np.int32)
    ci = np.array([k[1] for k in keys], dtype=np.int32)
    val = np.array([ent[k] for k in keys], dtype=np.float64)
    assert len(val) == g["nnz"]
    h = hashlib.sha256()
    h.update(ri.tobytes())
    h.update(ci.tobytes())
    h.update(val.tobytes())
    assert h.hexdigest() == g["sha256"]


def test_oracle_against_live_reference(nn, orc):
    """Where the reference's sources are present: lists, residuals and K11 bit for bit on a
    fresh case not used for the fixtures."""
    if orc.load_reference() is None:
        pytest.skip("reference sources not present")
    inp = nn.synth(1, 13, 99)
    p = inp["params"].copy()
    p.k_diss = 0.0
    p.vol_red = 0.3
    N = inp["N"]
    r = p.delta * (1 + 1e-5)
    lr, pr, cr, mr = orc.ref_build_clouds_hash(1024, r, p.dx * 10, p.dy * 10, p.dz * 10, inp["nodes"])
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    assert o.build_neighbours() == mr
    lo, po, co = o.clouds()
    assert np.array_equal(lo, lr) and np.array_equal(po, pr) and np.array_equal(co, cr)
    rng = np.random.default_rng(5)
    c = 0.05 + rng.random((4, N))
    phi = rng.standard_normal(N)
    Fr = orc.ref_residuals(p, inp["nodes"], pr, cr, c, phi, inp["phase0"], inp["bctypes"],
                           inp["bcvalues"], voln1rel=0.6)
    Fo = o.residuals(c, phi, inp["phase0"], voln1rel=0.6)
    assert np.array_equal(Fo[:4], Fr[:4]) and np.array_equal(Fo[4], Fr[10])


def test_oracle_capacity_error(nn, orc):
    inp = nn.synth(0, 12, 1)
    o = orc.Oracle.from_synth(inp)
    with pytest.raises(RuntimeError):
        o.build_neighbours(100)
    assert o.build_neighbours(123) == 123


def test_oracle_step_is_residual_update(nn, orc):
    """c^{n+1} = c^n - dt F(c^n, phi^n) off the Dirichlet set, with phi^n the converged
    potential (F11 = 0 on the unknowns)."""
    inp = nn.synth(1, 12, 4)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-13)
    c0, phi0, ph0, _ = o.state()
    phi, it, rel = o.solve_potential(c0, ph0, phi0)
    assert rel <= 1e-13
    F = o.residuals(c0, phi, ph0)
    o.forward(1)
    c1, phi1, ph1, _ = o.state()
    p = inp["params"]
    free = inp["bctypes"] == 1
    expect = np.maximum(c0 - p.dt * F[:4], p.c_floor)
    assert np.abs(c1[:, free] - expect[:, free]).max() <= 1e-15 * np.abs(expect).max()
    assert np.allclose(c1[:, ~free], 0.1)
    assert np.abs(phi1 - phi).max() <= 1e-12 * max(1e-300, np.abs(phi).max())
    # F11 vanishes on the unknowns of the solve
    assert np.abs(F[4][free & (ph0 == 0)]).max() <= 1e-10 * np.abs(F[4]).max() + 1e-14
