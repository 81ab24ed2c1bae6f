"""The reference's implicit time step with its complete model on the GPU (nnpp_chem_*: ten
species and the potential; main.cpp:640-922) against the oracle's restatement, whose eleven
tangents tests/test_oracle_chem_implicit.py pins to utils::NewtonMatrices and whose residual
is utils::Residuals' own (tests/test_chem_fixture.py): the same Newton iteration counts, the
states to the GMRES tolerance's rounding, identical masks, over three steps of a smooth state
with the data files' constants."""
import numpy as np
import pytest

import chem_case
import chem_state
from test_oracle_chem_implicit import GOLDEN, smooth_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    return nn


@pytest.mark.parametrize("kind,n,seed", [(1, 12, 5), (1, 20, 5), (0, 14, 2)])
def test_chem_steps_match_oracle(gpu, orc, kind, n, seed):
    nn = gpu
    g = np.load(GOLDEN)
    d2, dc, d11 = g["data2"].copy(), g["datac"], g["datac11"]
    nodes, phase, _, _, r, cell = chem_case.case_inputs(nn.synth, kind, n, seed, d2)
    inp = nn.synth(kind, n, seed)
    U = smooth_state(phase, d2)
    bt, bv = chem_state.bc11(inp, U, d2[7])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    ch = nn.ChemImplicit(nodes, clouds[:, :ml], lengths, bt, bv, d2, dc, d11)
    ch.set_state(U, phase, voln1rel=chem_case.VOLN1REL)
    p = nn.params_from_reference(d2, [dc[k] for k in range(4)], d11)
    o = orc.Oracle(p, nodes, inp["bctypes"], inp["bcvalues"], inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    Uo, pho = U.copy(), phase.copy()
    for s in range(3):
        ng, kg = ch.step(1)
        Uo, pho, no, ko = o.chem_implicit_step(Uo, pho, bt, bv, chem_case.VOLN1REL, d2, dc, d11)
        print("step %d: newton gpu %d oracle %d, gmres gpu %d oracle %d" % (s, ng, no, kg, ko))
        assert ng == no
        assert abs(kg - ko) <= max(4, 0.02 * ko)
    Ug, phg, v = ch.state()
    assert np.array_equal(phg, pho)
    for f in range(11):
        scale = np.linalg.norm(Uo[f]) or 1.0
        err = np.linalg.norm(Ug[f] - Uo[f]) / scale
        print("field %d rel-L2 %.2e" % (f + 1, err))
        assert err <= 1e-9, f
    assert v == chem_case.VOLN1REL  # the volume is refreshed every eighth step


def test_chem_rejects_bad_input(gpu):
    nn = gpu
    g = np.load(GOLDEN)
    d2, dc, d11 = g["data2"], g["datac"].copy(), g["datac11"]
    nodes, phase, _, _, r, cell = chem_case.case_inputs(nn.synth, 0, 10, 1, d2)
    inp = nn.synth(0, 10, 1)
    U = smooth_state(phase, d2)
    bt, bv = chem_state.bc11(inp, U, d2[7])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    ch = nn.ChemImplicit(nodes, clouds[:, :ml], lengths, bt, bv, d2, dc, d11)
    with pytest.raises(nn.NNPPError) as e:
        ch.step(1)  # no state yet
    assert e.value.status == 7
    dc[2, 3] = 0.5  # a kernel exponent s != 0
    with pytest.raises(nn.NNPPError) as e:
        nn.ChemImplicit(nodes, clouds[:, :ml], lengths, bt, bv, d2, dc, d11)
    assert e.value.status == 6


def test_chem_ten_steps_with_the_volume_update(gpu, orc):
    """Ten steps: the relative volume that sets BV is refreshed after the eighth
    (main.cpp:944-949, from the initial volume of main.cpp:474-480), on the GPU as in the
    oracle's steps driven here; states and phases agree after it."""
    nn = gpu
    g = np.load(GOLDEN)
    d2, dc, d11 = g["data2"].copy(), g["datac"], g["datac11"]
    nodes, phase, _, _, r, cell = chem_case.case_inputs(nn.synth, 1, 12, 5, d2)
    inp = nn.synth(1, 12, 5)
    U = smooth_state(phase, d2)
    bt, bv = chem_state.bc11(inp, U, d2[7])
    clouds, lengths, ml = nn.build_clouds_hash(1024, r, cell, cell, cell, nodes)
    ch = nn.ChemImplicit(nodes, clouds[:, :ml], lengths, bt, bv, d2, dc, d11)
    ch.set_state(U, phase, voln1rel=0.0)
    ch.step(10)
    Ug, phg, vg = ch.state()
    p = nn.params_from_reference(d2, [dc[k] for k in range(4)], d11)
    o = orc.Oracle(p, nodes, inp["bctypes"], inp["bcvalues"], inp["icvalues"], phase)
    o.build_neighbours(1024, r, (cell, cell, cell))
    csat = d2[8] / d2[7]
    vol0 = float(U[0][phase == 1].sum() - csat * (phase == 1).sum())
    Uo, pho, v = U.copy(), phase.copy(), 0.0
    for s in range(1, 11):
        Uo, pho, _, _ = o.chem_implicit_step(Uo, pho, bt, bv, v, d2, dc, d11)
        if s % 8 == 0:
            v = float(Uo[0][pho == 1].sum() - csat * (pho == 1).sum()) / vol0
    assert np.array_equal(phg, pho)
    assert abs(vg - v) <= 1e-12 * abs(v)
    for f in range(11):
        scale = np.linalg.norm(Uo[f]) or 1.0
        assert np.linalg.norm(Ug[f] - Uo[f]) <= 1e-9 * scale, f
