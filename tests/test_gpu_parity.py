"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle (which is
itself pinned to the reference's grid.h/utils.h, see test_oracle_pin.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# geometry kinds of nnpp_synth_fill with small sides
SMALL_CASES = [(0, 20), (1, 16), (2, 14), (3, 20), (4, 15)]


def _ref_rows_without_self(po, co, N):
    return [co[po[i] + 1:po[i + 1]] for i in range(N)]


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


@pytest.mark.parametrize("kind,n", SMALL_CASES)
def test_build_clouds_hash_reference_order_bit_exact(gpu, orc, kind, n):
    nn = gpu
    inp = nn.synth(kind, n, seed=11)
    p = inp["params"]
    r = p.delta * (1 + 1e-5)
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, p.dx * 10, p.dy * 10, p.dz * 10, inp["nodes"])
    o = orc.Oracle.from_synth(inp)
    ml_o = o.build_neighbours()
    lo, po, co = o.clouds()
    assert ml == ml_o
    assert np.array_equal(lengths, lo)
    # padded column-major matrix exactly as the reference's Eigen::MatrixXi
    expect = -np.ones((inp["N"], 1024), dtype=np.int32)
    for i in range(inp["N"]):
        expect[i, :lo[i]] = co[po[i]:po[i + 1]]
    assert np.array_equal(clouds, expect)


@pytest.mark.parametrize("name", ["lattice_block_20", "jittered_sphere_80", "screw_permuted_126"])
def test_full_size_clouds_bit_exact_vs_reference_digest(gpu, name):
    """8k, 512k and 2M workloads (the last randomly permuted): the GPU lists, neighbour
    order included, hash to the digest of the reference's own build_clouds_hash."""
    import hashlib
    import json
    import os
    from conftest import GOLDEN_DIR
    nn = gpu
    with open(os.path.join(GOLDEN_DIR, "clouds.json")) as f:
        g = json.load(f)[name]
    inp = nn.synth(g["kind"], g["n_side"], g["seed"])
    sim = nn.Simulation.from_synth(inp)
    _, lengths, ml = sim.build_neighbours()
    ptr, cols = sim.neighbours_csr()
    N = inp["N"]
    full = np.empty(len(cols) + N, dtype=np.int32)
    self_pos = ptr[:-1] + np.arange(N)
    full[self_pos] = np.arange(N, dtype=np.int32)
    mask = np.ones(len(full), dtype=bool)
    mask[self_pos] = False
    full[mask] = cols
    h = hashlib.sha256()
    h.update(lengths.astype(np.int32).tobytes())
    h.update(full.tobytes())
    assert ml == g["max_len"] and len(cols) + N == g["nnz"]
    assert h.hexdigest() == g["sha256"]


@pytest.mark.parametrize("cell_factor", [10.0, 1.0, 0.7])
def test_build_other_cell_sizes(gpu, orc, cell_factor):
    """Cells smaller than the horizon exercise the multi-cell scan (grid.h:157-167)."""
    nn = gpu
    inp = nn.synth(1, 14, seed=2)
    p = inp["params"]
    r = p.delta * (1 + 1e-5)
    cell = p.dx * cell_factor
    _, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, inp["nodes"], want_clouds=False)
    o = orc.Oracle.from_synth(inp)
    ml_o = o.build_neighbours(1024, r, (cell, cell, cell))
    lo, po, co = o.clouds()
    assert ml == ml_o and np.array_equal(lengths, lo)
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours(1024, r, (cell, cell, cell))
    ptr, cols = sim.neighbours_csr()
    rows = _ref_rows_without_self(po, co, inp["N"])
    assert np.array_equal(cols, np.concatenate(rows))


def test_canonical_order_same_sets(gpu, orc):
    nn = gpu
    inp = nn.synth(2, 14, seed=5)
    sim_r = nn.Simulation.from_synth(inp)
    sim_r.build_neighbours(order_mode=nn.ORDER_REFERENCE)
    sim_c = nn.Simulation.from_synth(inp)
    sim_c.build_neighbours(order_mode=nn.ORDER_CANONICAL)
    pr, cr = sim_r.neighbours_csr()
    pc, cc = sim_c.neighbours_csr()
    assert np.array_equal(pr, pc)
    for i in range(inp["N"]):
        a, b = cr[pr[i]:pr[i + 1]], cc[pc[i]:pc[i + 1]]
        assert np.array_equal(np.sort(a), np.sort(b))


def test_capacity_error_matches_reference(gpu, orc):
    """grid.h:187-189 throws when a list does not fit; the C ABI returns NNPP_ERR_CAPACITY."""
    nn = gpu
    inp = nn.synth(0, 12, seed=1)
    p = inp["params"]
    with pytest.raises(nn.NNPPError) as ei:
        nn.build_clouds_hash(64, p.delta * (1 + 1e-5), p.dx * 10, p.dy * 10, p.dz * 10, inp["nodes"])
    assert ei.value.status == 2
    o = orc.Oracle.from_synth(inp)
    with pytest.raises(RuntimeError):
        o.build_neighbours(64)
    # exactly enough room passes
    _, lengths, ml = nn.build_clouds_hash(123, p.delta * (1 + 1e-5), p.dx * 10, p.dy * 10, p.dz * 10,
                                          inp["nodes"], want_clouds=False)
    assert ml == 123


def _random_state(rng, inp, scale_phi=0.3):
    N = inp["N"]
    c = 0.05 + rng.random((4, N))
    phi = rng.standard_normal(N) * scale_phi
    ph = inp["phase0"].copy()
    return c, phi, ph


@pytest.mark.parametrize("kind,n", [(0, 16), (1, 16), (2, 14)])
def test_residuals_fp64_and_mixed(gpu, orc, kind, n):
    nn = gpu
    rng = np.random.default_rng(kind)
    inp = nn.synth(kind, n, seed=3)
    p = inp["params"].copy()
    p.vol_red = 0.5
    sim = nn.Simulation(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    sim.build_neighbours()
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    c, phi, ph = _random_state(rng, inp)
    Fo = o.residuals(c, phi, ph, voln1rel=0.25)
    F64 = sim.residuals(c, phi, ph, voln1rel=0.25, precision=nn.FP64)
    F32 = sim.residuals(c, phi, ph, voln1rel=0.25, precision=nn.MIXED)
    for k in range(5):
        scale = np.abs(Fo[k]).max()
        assert np.abs(F64[k] - Fo[k]).max() <= 1e-12 * scale, k
    # FP32 bond sums with compensated reduction: per-node error relative to the row scale
    for k in range(4):
        scale = np.abs(Fo[k]).max()
        assert np.abs(F32[k] - Fo[k]).max() <= 2e-5 * scale, k
    # the mixed path's potential residual F11: FP64 arithmetic on the potential held as an
    # FP32 pair (hi + lo, ~2^-48 of the value)
    scale = np.abs(Fo[4]).max()
    assert np.abs(F32[4] - Fo[4]).max() <= 1e-10 * scale


@pytest.mark.parametrize("prec", [0, 1])
def test_solve_potential(gpu, orc, prec):
    nn = gpu
    rng = np.random.default_rng(7)
    inp = nn.synth(1, 18, seed=4)
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.set_solver(1e-10)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-13)
    c, _, ph = _random_state(rng, inp)
    phi_o, it_o, rel_o = o.solve_potential(c, ph)
    phi_g, it_g, rel_g = sim.solve_potential(c, ph, precision=prec)
    assert rel_g <= 1e-10
    err = np.linalg.norm(phi_g - phi_o) / np.linalg.norm(phi_o)
    assert err < 1e-8, err
    # the reference's F11 (utils.h:798-841), evaluated by the oracle at the GPU solution,
    # vanishes on the unknowns (non-Dirichlet liquid rows) to the solve's tolerance
    F = o.residuals(c, phi_g, ph)
    rows = (inp["bctypes"] == 1) & (ph == 0)
    lam = (1.0 / (inp["params"].K_phi * inp["params"].sigma)) * inp["params"].F * inp["params"].CSolid
    b = lam * (np.array(list(inp["params"].z)) @ c)
    assert np.linalg.norm(F[4][rows]) <= 2e-10 * np.linalg.norm(b[rows])


def test_forward_fp64_lattice_block_masks_bit_exact(gpu, orc):
    """Plain FP64 lattice workload, 1000 steps: final mask and every flip step identical to
    the oracle; fields to rounding."""
    nn = gpu
    inp = nn.synth(0, 20, seed=0)
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.set_solver(1e-12)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-13)
    for _ in range(4):
        sim.forward(250, nn.FP64)
        o.forward(250)
    c_g, phi_g, ph_g = sim.state()
    c_o, phi_o, ph_o, fs_o = o.state()
    assert np.array_equal(ph_g, ph_o)
    assert np.array_equal(sim.flip_steps(), fs_o)
    assert (fs_o > 0).sum() == 1000  # the block dissolves completely
    assert np.linalg.norm(c_g - c_o) / np.linalg.norm(c_o) < 1e-10
    assert np.linalg.norm(phi_g - phi_o) / np.linalg.norm(phi_o) < 1e-8
    dg = sim.diagnostics()
    do = o.diagnostics()
    assert dg["solid_count"] == do["solid_count"] == 0
    assert abs(dg["mg_mass_lost"] - do["mg_mass_lost"]) <= 1e-10 * abs(do["mg_mass_lost"])


def test_forward_mixed_vs_oracle(gpu, orc):
    nn = gpu
    inp = nn.synth(1, 20, seed=9)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-13)
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.forward(200, nn.MIXED)
    o.forward(200)
    c_g, phi_g, ph_g = sim.state()
    c_o, phi_o, ph_o, _ = o.state()
    assert np.linalg.norm(c_g - c_o) / np.linalg.norm(c_o) <= 1e-5
    assert np.linalg.norm(phi_g - phi_o) / np.linalg.norm(phi_o) <= 1e-5
    assert np.array_equal(ph_g, ph_o)


def test_step_host_matches_forward(gpu):
    nn = gpu
    inp = nn.synth(1, 14, seed=1)
    a = nn.Simulation.from_synth(inp)
    a.build_neighbours()
    b = nn.Simulation.from_synth(inp)
    b.build_neighbours()
    c, phi, ph = b.state()
    for _ in range(5):
        c, phi, ph = b.step_host(c, ph, precision=nn.FP64)
    a.forward(5, nn.FP64)
    ca, phia, pha = a.state()
    assert np.array_equal(ph, pha)
    assert np.abs(c - ca).max() <= 1e-13 * np.abs(ca).max()
    assert np.abs(phi - phia).max() <= 1e-10 * max(np.abs(phia).max(), 1e-300)


def test_state_roundtrip_and_errors(gpu):
    nn = gpu
    inp = nn.synth(0, 10, seed=1)
    sim = nn.Simulation.from_synth(inp)
    with pytest.raises(nn.NNPPError) as ei:
        sim.forward(1)
    assert ei.value.status == 7  # steps before the neighbour build
    sim.build_neighbours()
    c, phi, ph = sim.state()
    sim.set_state(c * 1.5, phi, ph)
    c2, phi2, ph2 = sim.state()
    assert np.array_equal(c2, c * 1.5) and np.array_equal(ph2, ph)
    c3 = c.copy()
    c3[0, int(np.argmax(inp["bctypes"] == 1))] = np.nan
    sim.set_state(c3, phi, ph)
    with pytest.raises(nn.NNPPError) as ei:
        sim.forward(2, nn.FP64)
    assert ei.value.status == 3


def test_ensemble_matches_individual_runs(gpu):
    """Uneven instances with their own parameters in one batched launch give the same
    states as each instance run alone."""
    nn = gpu
    cases = [nn.synth(4, 14, 1), nn.synth(4, 20, 2), nn.synth(4, 17, 3), nn.synth(1, 12, 4)]
    sims = []
    for inp in cases:
        s = nn.Simulation.from_synth(inp)
        s.build_neighbours()
        s.set_solver(1e-12)
        sims.append(s)
    ens = nn.Ensemble(sims)
    ens.forward(30, nn.FP64)
    T, W = ens.tuning()
    assert T in (2, 4, 8) and W in (4, 8, 16)
    for inp, s in zip(cases, sims):
        alone = nn.Simulation.from_synth(inp)
        alone.build_neighbours()
        alone.set_solver(1e-12)
        alone.forward(30, nn.FP64)
        c_e, phi_e, ph_e = s.state()
        c_a, phi_a, ph_a = alone.state()
        assert np.array_equal(ph_e, ph_a)
        assert np.abs(c_e - c_a).max() <= 1e-11 * np.abs(c_a).max()
        assert np.abs(phi_e - phi_a).max() <= 1e-8 * max(np.abs(phi_a).max(), 1e-30)
        assert s.diagnostics()["steps_done"] == 30
    # mixed precision through the same ensemble, then continue one member alone
    ens.forward(10, nn.MIXED)
    sims[0].forward(2, nn.MIXED)
    assert sims[0].diagnostics()["steps_done"] == 42
    ens.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_warm_start_modes_agree_and_history_saves_iterations(gpu, prec):
    """The warm start changes only the iteration count: after 60 steps every mode gives the
    same state to the solver tolerance, and the history projection needs fewer CG
    iterations than the linear extrapolation."""
    nn = gpu
    inp = nn.synth(1, 24, seed=4)
    out = {}
    for mode in (0, 1, 6):
        sim = nn.Simulation.from_synth(inp)
        sim.build_neighbours()
        sim.set_warm_start(mode)
        sim.set_solver(1e-11)
        sim.forward(60, prec)
        out[mode] = (sim.state(), sim.diagnostics())
    (c1, phi1, ph1), d1 = out[1]
    for mode in (0, 6):
        (c, phi, ph), d = out[mode]
        assert np.array_equal(ph, ph1)
        assert np.linalg.norm(c - c1) <= 1e-8 * np.linalg.norm(c1)
        assert np.linalg.norm(phi - phi1) <= 1e-8 * np.linalg.norm(phi1)
        assert d["cg_not_converged"] == 0
    assert out[6][1]["cg_iterations_total"] < 0.8 * out[1][1]["cg_iterations_total"]
    assert out[1][1]["cg_iterations_total"] < out[0][1]["cg_iterations_total"]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n", [24, 48])
def test_preconditioners_agree_and_two_level_saves_iterations(gpu, orc, prec, n):
    """The two-level preconditioner changes only the iteration count: both preconditioners
    reach the oracle's state (to 1e-9 in FP64, the mixed tolerance in mixed precision), and
    the coarse correction needs fewer CG iterations.  n = 48 has more bins than coarse
    unknowns, so aggregates of 2 x 2 x 2 bins are formed."""
    nn = gpu
    inp = nn.synth(1, n, seed=9)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-13)
    o.forward(30)
    c_o, phi_o, ph_o, _ = o.state()
    out = {}
    for kind in (nn.PRECOND_JACOBI, nn.PRECOND_TWO_LEVEL):
        sim = nn.Simulation.from_synth(inp)
        sim.build_neighbours()
        sim.set_preconditioner(kind)
        k, cn, every, _ = sim.preconditioner()
        assert k == kind and (cn > 0) == (kind == nn.PRECOND_TWO_LEVEL) and every == 64
        sim.forward(30, prec)
        out[kind] = (sim.state(), sim.diagnostics(), cn)
    tol = 1e-9 if prec == nn.FP64 else 1e-5
    for kind, ((c, phi, ph), d, cn) in out.items():
        assert np.array_equal(ph, ph_o)
        assert np.linalg.norm(c - c_o) <= tol * np.linalg.norm(c_o)
        assert np.linalg.norm(phi - phi_o) <= tol * np.linalg.norm(phi_o)
        assert d["cg_not_converged"] == 0
    it_j = out[nn.PRECOND_JACOBI][1]["cg_iterations_total"]
    it_c = out[nn.PRECOND_TWO_LEVEL][1]["cg_iterations_total"]
    assert it_c < 0.8 * it_j, (it_c, it_j)


def test_two_level_is_reproducible_and_follows_set_state(gpu):
    """Two runs from the same state give identical bits; a new state (set_state) rebuilds
    the coarse operator, so a run after set_state equals a run of a fresh handle.  The
    configuration is pinned (the autotuner's choice changes the summation order)."""
    nn = gpu
    inp = nn.synth(1, 32, seed=5)

    def make():
        s = nn.Simulation.from_synth(inp)
        s.build_neighbours()
        s.set_tuning(4, 8, 0)
        return s

    sims = []
    for _ in range(2):
        sim = make()
        sim.forward(20, nn.MIXED)
        sims.append(sim.state())
    for a, b in zip(*sims):
        assert np.array_equal(a, b)
    sim = make()
    sim.forward(20, nn.MIXED)
    c, phi, ph = sim.state()
    fresh = make()
    fresh.set_state(c, phi, ph)
    fresh.forward(10, nn.MIXED)
    sim.set_state(c, phi, ph)
    sim.forward(10, nn.MIXED)
    for a, b in zip(sim.state(), fresh.state()):
        assert np.array_equal(a, b)


def test_preconditioner_rejects_bad_kind(gpu):
    nn = gpu
    inp = nn.synth(1, 12, seed=4)
    sim = nn.Simulation.from_synth(inp)
    for bad in ((2, 64), (1, -1)):
        with pytest.raises(nn.NNPPError) as e:
            sim.set_preconditioner(*bad)
        assert e.value.status == 1


@pytest.mark.parametrize("prec", [0, 1])
def test_coarse_rebuild_follows_dissolution(gpu, orc, prec):
    """The implant dissolves between steps 35 and 40 (k_diss = 0.1): with a refresh period of
    4 steps the coarse operator is rebuilt after the flip; with period 0 it keeps the initial
    phases.  Both runs and a Jacobi run reach the oracle's state."""
    nn = gpu
    inp = nn.synth(1, 12, 5)
    p = inp["params"].copy()
    p.switch_width = 0.01
    p.k_diss = 0.1
    args = (p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o = orc.Oracle(*args)
    o.build_neighbours()
    o.set_solver(1e-13)
    o.forward(60)
    c_o, phi_o, ph_o, _ = o.state()
    assert (ph_o != inp["phase0"]).sum() > 0
    tol = 1e-9 if prec == nn.FP64 else 1e-5
    rebuilds = {}
    for kind, every in ((nn.PRECOND_TWO_LEVEL, 4), (nn.PRECOND_TWO_LEVEL, 0), (nn.PRECOND_JACOBI, 4)):
        sim = nn.Simulation(*args)
        sim.build_neighbours()
        sim.set_preconditioner(kind, every)
        sim.forward(60, prec)
        c, phi, ph = sim.state()
        assert np.array_equal(ph, ph_o)
        assert np.linalg.norm(c - c_o) <= tol * np.linalg.norm(c_o)
        assert np.linalg.norm(phi - phi_o) <= tol * np.linalg.norm(phi_o)
        assert sim.diagnostics()["cg_not_converged"] == 0
        rebuilds[(kind, every)] = sim.preconditioner()[3]
    assert rebuilds[(nn.PRECOND_TWO_LEVEL, 0)] == 1
    assert rebuilds[(nn.PRECOND_TWO_LEVEL, 4)] >= 2
    assert rebuilds[(nn.PRECOND_JACOBI, 4)] == 0


@pytest.mark.parametrize("prec", [0, 1])
def test_nodes_turned_liquid_start_from_their_neighbours_potential(gpu, prec):
    """After the step in which a node turns liquid, its potential (the next solve's guess) is a
    weighted mean of the potentials of its neighbours that were liquid before that step: it
    lies between their extremes, not at the solid's zero."""
    nn = gpu
    inp = nn.synth(1, 12, 5)
    p = inp["params"].copy()
    p.switch_width = 0.01
    p.k_diss = 0.1
    sim = nn.Simulation(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    sim.build_neighbours()
    ptr, cols = sim.neighbours_csr()
    phi_dir = (np.asarray(inp["bctypes"]) == 0) & (np.asarray(inp["bcvalues"])[4] != -1)
    checked = 0
    for step in range(1, 61):
        _, _, ph0 = sim.state()
        sim.forward(1, prec)
        _, phi, ph1 = sim.state()
        flipped = np.nonzero((ph0 != 0) & (ph1 == 0))[0]
        for a in flipped:
            if phi_dir[a]:
                continue
            nb = cols[ptr[a]:ptr[a + 1]]
            nb = nb[(ph0[nb] == 0)]
            if nb.size == 0:
                continue
            lo, hi = phi[nb].min(), phi[nb].max()
            span = max(hi - lo, 1e-12 * max(abs(lo), abs(hi), 1.0))
            assert lo - 1e-9 * span <= phi[a] <= hi + 1e-9 * span
            assert phi[a] != 0.0 or (lo <= 0.0 <= hi)
            checked += 1
    assert checked > 0


def test_refinement_settings(gpu):
    """A looser inner reduction per FP32 sweep costs refinement sweeps, not accuracy; bad
    settings are rejected."""
    nn = gpu
    inp = nn.synth(1, 16, 3)
    out = {}
    for rel in (1e-4, 1e-2):
        sim = nn.Simulation.from_synth(inp)
        sim.build_neighbours()
        sim.set_refinement(rel, 30)
        sim.forward(20, nn.MIXED)
        d = sim.diagnostics()
        out[rel] = (sim.state(), d["outer_iterations_total"], d["cg_not_converged"])
    (s4, o4, nc4), (s2, o2, nc2) = out[1e-4], out[1e-2]
    assert nc4 == 0 and nc2 == 0
    assert o2 > o4
    for a, b in zip(s4[:2], s2[:2]):
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(a)
    sim = nn.Simulation.from_synth(inp)
    for bad in ((0.0, 30), (1.0, 30), (1e-4, 0)):
        with pytest.raises(nn.NNPPError) as e:
            sim.set_refinement(*bad)
        assert e.value.status == 1


def test_warm_start_rejects_bad_history(gpu):
    nn = gpu
    inp = nn.synth(1, 12, seed=4)
    sim = nn.Simulation.from_synth(inp)
    with pytest.raises(nn.NNPPError) as e:
        sim.set_warm_start(7)
    assert e.value.status == 1


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7, 8])
def test_cg_operator_variants_vs_oracle(gpu, orc, variant):
    """Every FP32 CG operator (L1/L2 gathers; bulk-copy staged; shared-memory windows; with
    and without L2 prefetch of the operator stream; the halo-staged operator with recomputed
    weights) reaches the oracle's state to the mixed-precision tolerance, configuration
    pinned."""
    nn = gpu
    inp = nn.synth(1, 20, seed=11)
    o = orc.Oracle.from_synth(inp)
    o.build_neighbours()
    o.set_solver(1e-13)
    o.forward(100)
    c_o, phi_o, ph_o, _ = o.state()
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.set_tuning(8, 8, variant)
    sim.forward(100, nn.MIXED)
    assert sim.tuning() == (8, 8, variant)
    c_g, phi_g, ph_g = sim.state()
    assert np.array_equal(ph_g, ph_o)
    assert np.linalg.norm(c_g - c_o) / np.linalg.norm(c_o) <= 1e-5
    assert np.linalg.norm(phi_g - phi_o) / np.linalg.norm(phi_o) <= 1e-5
    assert sim.diagnostics()["cg_not_converged"] == 0


@pytest.mark.parametrize("n,T", [(12, 2), (12, 4), (24, 4), (24, 8)])
def test_transport_variants_give_the_same_bits(gpu, n, T):
    """The FP32 transport with each tile's halo records staged in shared memory (form 1) and
    with the records gathered from L1/L2 (0): the same sums in the same order, so the same
    states bit for bit, at several tile lengths, through a fast dissolution (phases flip on
    the small lattice)."""
    nn = gpu
    inp = nn.synth(1, n, 5)
    p = inp["params"].copy()
    p.switch_width = 0.01
    p.k_diss = 0.1
    out = []
    for variant in range(2):
        sim = nn.Simulation(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
        sim.build_neighbours()
        sim.set_tuning(T, 8, 0)
        sim.set_transport_variant(variant)
        sim.forward(60, nn.MIXED)
        out.append((sim.state(), sim.diagnostics()))
    s0, d0 = out[0]
    if n == 12:
        assert d0["solid_count"] < int((np.asarray(inp["phase0"]) != 0).sum())
    for s1, d1 in out[1:]:
        for a, b in zip(s0, s1):
            assert np.array_equal(a, b)
        assert d0["solid_count"] == d1["solid_count"]
        assert abs(d0["mg_mass_lost"] - d1["mg_mass_lost"]) <= 1e-12 * abs(d0["mg_mass_lost"])
    for bad in (-1, 2):
        with pytest.raises(nn.NNPPError) as e:
            sim.set_transport_variant(bad)
        assert e.value.status == 1


def test_set_tuning_rejects_bad_configuration(gpu):
    nn = gpu
    inp = nn.synth(1, 12, seed=4)
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    for bad in ((3, 8, 0), (8, 5, 0), (8, 8, 9), (8, 8, -1)):
        with pytest.raises(nn.NNPPError) as e:
            sim.set_tuning(*bad)
        assert e.value.status == 1


def test_time_kernel_parts_leave_the_state(gpu):
    """nnpp_time_kernel times the split update's three kernels one by one on a single
    instance with the coarse space (ids 4-6), restores the state afterwards, and rejects
    them without a coarse space and out-of-range ids."""
    nn = gpu
    inp = nn.synth(1, 16, seed=3)
    sim = nn.Simulation.from_synth(inp)
    sim.build_neighbours()
    sim.set_tuning(4, 8, 0)
    sim.forward(3, nn.MIXED)
    before = sim.state()
    for kid in range(7):
        assert sim.time_kernel(kid, nn.MIXED, reps=3) > 0.0
    for a, b in zip(before, sim.state()):
        assert np.array_equal(a, b)
    ref = nn.Simulation.from_synth(inp)
    ref.build_neighbours()
    ref.set_tuning(4, 8, 0)
    ref.forward(3, nn.MIXED)
    sim.forward(2, nn.MIXED)
    ref.forward(2, nn.MIXED)
    for a, b in zip(sim.state(), ref.state()):
        assert np.array_equal(a, b)
    jac = nn.Simulation.from_synth(inp)
    jac.build_neighbours()
    jac.set_preconditioner(nn.PRECOND_JACOBI)
    jac.forward(1, nn.MIXED)
    with pytest.raises(nn.NNPPError) as e:
        jac.time_kernel(5, nn.MIXED, reps=1)
    assert e.value.status == 1
    with pytest.raises(nn.NNPPError) as e:
        sim.time_kernel(7, nn.MIXED, reps=1)
    assert e.value.status == 1
