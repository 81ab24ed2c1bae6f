"""The ten-species residual fixture (CPU): its control vectors are the reference data files'
shapes, its cases' inputs are reproducible here, and, where the reference's sources are
present, the reference compiled here still gives the stored residuals bit for bit."""
import os

import numpy as np
import pytest

import chem_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "chemistry.npz")


def test_fixture_shapes_and_inputs(orc):
    g = np.load(GOLDEN)
    assert g["data2"].shape == (51,) and g["datac"].shape == (10, 7) and g["datac11"].shape == (4,)
    for kind, n, seed in chem_case.CASES:
        nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(orc.synth, kind, n, seed, g["data2"])
        N = nodes.shape[1]
        for which in ("F", "Freactive"):
            F = g["kind%d_n%d_seed%d_%s" % (kind, n, seed, which)]
            assert F.shape == (11, N) and np.isfinite(F).all()
        assert (phase == 1).any() and (phase == 0).any()


@pytest.mark.parametrize("kind,n,seed", chem_case.CASES)
def test_oracle_full_residual_matches_reference_bit_for_bit(orc, kind, n, seed):
    """The oracle's restatement of the ten-species residual gives the reference's bits, with
    the physical constants and with the reactive ones; clouds from the oracle's neighbour
    build (the reference's order)."""
    g = np.load(GOLDEN)
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(orc.synth, kind, n, seed, g["data2"])
    inp = orc.synth(kind, n, seed)
    o = orc.Oracle(inp["params"], nodes, inp["bctypes"], inp["bcvalues"], inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    lengths, ptr, cols = o.clouds()
    for which, d2 in (("F", g["data2"]), ("Freactive", chem_case.reactive_data2(g["data2"]))):
        F = orc.residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, g["datac"], g["datac11"])
        assert np.array_equal(F, g["kind%d_n%d_seed%d_%s" % (kind, n, seed, which)]), which


def test_reference_reproduces_fixture(orc):
    if orc.load_reference() is None:
        pytest.skip("reference sources not present")
    g = np.load(GOLDEN)
    kind, n, seed = chem_case.CASES[0]
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(orc.synth, kind, n, seed, g["data2"])
    lo, po, co, ml = orc.ref_build_clouds_hash(1024, r, cell, cell, cell, nodes)
    for which, d2 in (("F", g["data2"]), ("Freactive", chem_case.reactive_data2(g["data2"]))):
        F = orc.ref_residuals_full(nodes, po, co, Un1, Un, phase, chem_case.VOLN1REL, d2, g["datac"], g["datac11"])
        assert np.array_equal(F, g["kind%d_n%d_seed%d_%s" % (kind, n, seed, which)])


def test_oracle_general_exponents_match_reference(orc):
    """Exponents 3 + 2 s that differ between species and terms: the oracle's restatement
    against the reference compiled here, bit for bit (skipped where the reference's sources
    are absent)."""
    g = np.load(GOLDEN)
    dc = g["datac"].copy()
    dc[:, 3] = np.linspace(0.0, 0.9, 10)
    dc[:, 4] = 0.5
    d11 = g["datac11"].copy()
    d11[2] = 0.25
    d2 = chem_case.reactive_data2(g["data2"])
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(orc.synth, 0, 12, 3, g["data2"])
    inp = orc.synth(0, 12, 3)
    o = orc.Oracle(inp["params"], nodes, inp["bctypes"], inp["bcvalues"], inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    lengths, ptr, cols = o.clouds()
    Fr = orc.ref_residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    if Fr is None:
        pytest.skip("the reference's sources are not compiled here")
    F = orc.residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    assert np.array_equal(F, Fr)
