"""The reference's complete residual on the GPU (nnpp_residuals_full: ten species, their
reactions, the interface's H+ source, the potential; utils.h:29-842) against the reference's
own utils::Residuals on the same inputs (tests/golden/chemistry.npz, made by
tests/golden/make_golden.py --only-chemistry from the reference compiled here), with the
physical constants of the reference's data files and with constants that put every reaction
term at the transport terms' size."""
import os

import numpy as np
import pytest

import chem_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "chemistry.npz")


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


@pytest.mark.parametrize("kind,n,seed", chem_case.CASES)
@pytest.mark.parametrize("which", ["F", "Freactive"])
def test_residuals_full_match_reference(gpu, gold, kind, n, seed, which):
    nn = gpu
    d2, dc, d11 = gold["data2"], gold["datac"], gold["datac11"]
    if which == "Freactive":
        d2 = chem_case.reactive_data2(d2)
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(nn.synth, kind, n, seed, gold["data2"])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    F = nn.residuals_full(nodes, clouds[:, :ml], lengths, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    Fr = gold["kind%d_n%d_seed%d_%s" % (kind, n, seed, which)]
    assert F.shape == Fr.shape
    for k in range(11):
        scale = np.abs(Fr[k]).max()
        assert np.abs(F[k] - Fr[k]).max() <= 1e-12 * scale, k
        # the potential row is zero exactly where the reference leaves it zero
        if k == 10:
            assert np.array_equal(F[k] == 0.0, Fr[k] == 0.0)


def test_residuals_full_rejects_bad_input(gpu, gold):
    nn = gpu
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(nn.synth, 0, 12, 3, gold["data2"])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    bad = clouds[:, :ml].copy()
    bad[5, 1] = nodes.shape[1]  # a neighbour index past the last node
    with pytest.raises(nn.NNPPError) as e:
        nn.residuals_full(nodes, bad, lengths, Un1, Un, phase, 0.3, gold["data2"], gold["datac"], gold["datac11"])
    assert e.value.status == 1
    d2 = gold["data2"].copy()
    d2[2] = 0.0  # dt
    with pytest.raises(nn.NNPPError) as e:
        nn.residuals_full(nodes, clouds[:, :ml], lengths, Un1, Un, phase, 0.3, d2, gold["datac"], gold["datac11"])
    assert e.value.status == 1


def _oracle_clouds(clouds, lengths, ml):
    ptr = np.zeros(lengths.size + 1, dtype=np.int64)
    ptr[1:] = np.cumsum(lengths)
    cols = clouds[:, :ml][np.arange(ml)[None, :] < lengths[:, None]].astype(np.int32)
    return ptr, cols


def _assert_close(F, Fr):
    for k in range(11):
        scale = np.abs(Fr[k]).max()
        assert np.abs(F[k] - Fr[k]).max() <= 1e-12 * scale, k
    assert np.array_equal(F[10] == 0.0, Fr[10] == 0.0)


@pytest.mark.parametrize("reactive", [False, True])
def test_residuals_full_match_oracle_at_64k(gpu, orc, gold, reactive):
    """The 40^3 lattice (64,000 nodes, ~100 bonds a node) against the oracle's restatement,
    which gives the reference's bits on the fixture cases."""
    nn = gpu
    d2 = chem_case.reactive_data2(gold["data2"]) if reactive else gold["data2"]
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(nn.synth, 1, 40, 1, gold["data2"])
    clouds, lengths, ml = nn.build_clouds_hash(160, r, cell, cell, cell, nodes)
    F = nn.residuals_full(nodes, clouds[:, :ml], lengths, Un1, Un, phase, chem_case.VOLN1REL, d2,
                          gold["datac"], gold["datac11"])
    ptr, cols = _oracle_clouds(clouds, lengths, ml)
    Fr = orc.residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, gold["datac"],
                            gold["datac11"])
    _assert_close(F, Fr)


def test_residuals_full_general_exponents(gpu, orc, gold):
    """Exponents 3 + 2 s that differ between species, terms and the potential (s_k1, s_k2,
    s111 not zero): the kernel's per-term powers against the oracle's."""
    nn = gpu
    dc = gold["datac"].copy()
    dc[:, 3] = np.linspace(0.0, 0.9, 10)   # s_k1
    dc[:, 4] = 0.5                        # s_k2
    d11 = gold["datac11"].copy()
    d11[2] = 0.25                         # s111
    d2 = chem_case.reactive_data2(gold["data2"])
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(nn.synth, 0, 16, 2, gold["data2"])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    F = nn.residuals_full(nodes, clouds[:, :ml], lengths, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    ptr, cols = _oracle_clouds(clouds, lengths, ml)
    Fr = orc.residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    _assert_close(F, Fr)


def test_residuals_full_species_without_liquid_diffusion(gpu, orc, gold):
    """A species whose liquid diffusivity is zero (its liquid-liquid bonds carry nothing, the
    others still do): the kernel's per-class factors against the oracle's."""
    nn = gpu
    dc = gold["datac"].copy()
    dc[3, 2] = 0.0   # D_liquid of species 4
    dc[6, 6] = 0.0   # K_7prop2: species 7 without migration
    d2 = chem_case.reactive_data2(gold["data2"])
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(nn.synth, 1, 16, 4, gold["data2"])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    F = nn.residuals_full(nodes, clouds[:, :ml], lengths, Un1, Un, phase, chem_case.VOLN1REL, d2, dc,
                          gold["datac11"])
    ptr, cols = _oracle_clouds(clouds, lengths, ml)
    Fr = orc.residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, gold["datac11"])
    _assert_close(F, Fr)


def test_residuals_full_512k_matches_oracle(gpu, orc, gold):
    """The benchmark's chemistry workload itself (the 80^3 lattice, 512,000 nodes, 53.9M bonds,
    the reference's physical constants) against the oracle's restatement."""
    nn = gpu
    d2, dc, d11 = gold["data2"], gold["datac"], gold["datac11"]
    nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(nn.synth, 1, 80, 1, d2)
    clouds, lengths, ml = nn.build_clouds_hash(160, r, cell, cell, cell, nodes)
    F = nn.residuals_full(nodes, clouds[:, :ml], lengths, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    ptr, cols = _oracle_clouds(clouds, lengths, ml)
    del clouds
    Fr = orc.residuals_full(nodes, ptr, cols, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
    _assert_close(F, Fr)
