"""Host-side checks of the C ABI library (no GPU needed): it loads, exports every entry
point include/nnpp_gb300.h declares, reports the absence of a GPU as an error, maps the
reference's control vectors, and generates deterministic inputs."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_DIR, ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "nnpp_gb300.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nnpp_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(nn):
    L = nn.lib()
    names = _declared()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    # and the binding wraps all of them
    assert set(names) <= set(nn.exported_symbols())


def test_abi_version_and_last_error(nn):
    L = nn.lib()
    assert L.nnpp_abi_version() == 1
    assert isinstance(L.nnpp_last_error(), bytes)


def test_no_gpu_is_an_error_not_a_fallback(nn):
    if nn.device_count() > 0:
        pytest.skip("a GPU is present")
    inp = nn.synth(0, 6, 0)
    with pytest.raises(nn.NNPPError) as ei:
        nn.Simulation.from_synth(inp)
    assert ei.value.status == 5
    with pytest.raises(nn.NNPPError) as ei:
        p = inp["params"]
        nn.build_clouds_hash(1024, p.delta, p.dx * 10, p.dy * 10, p.dz * 10, inp["nodes"])
    assert ei.value.status == 5


def test_params_from_reference_control_vectors(nn):
    with open(os.path.join(GOLDEN_DIR, "params.json")) as f:
        g = json.load(f)
    d2 = g["NNPP.data2"]
    dc = [g["NNPP.datac%d" % k] for k in range(1, 5)]
    d11 = g["NNPP.datac11"]
    p = nn.params_from_reference(d2, dc, d11, k_diss=0.05, switch_width=0.0)
    # utils.h:2346-2395
    assert (p.dt, p.dx, p.dy, p.dz, p.delta) == tuple(d2[2:7])
    assert (p.CSolid, p.CSat) == (d2[7], d2[8])
    assert (p.T, p.R, p.F, p.vol_red) == (d2[47], d2[48], d2[49], d2[50])
    for k in range(4):  # utils.h:2397-2423
        assert (p.z[k], p.D_solid[k], p.D_liquid[k], p.s1[k], p.s2[k], p.K1[k], p.K2[k]) == tuple(dc[k])
    assert (p.sigma, p.s_phi, p.K_phi) == tuple(d11[1:4])  # utils.h:2480-2483
    assert p.c_floor == 1e-8 / d2[7]  # main.cpp:806
    assert p.sub_step_no == 8  # main.cpp:39
    # K_prop1 = 3/(pi delta^2), K_prop2 = 1/(pi delta^2) in the reference's data
    assert abs(p.K1[0] - 3 / (np.pi * p.delta ** 2)) <= 1e-12 * p.K1[0]
    assert abs(p.K2[0] - 1 / (np.pi * p.delta ** 2)) <= 1e-12 * p.K2[0]


def test_params_from_reference_rejects_null(nn):
    L = nn.lib()
    st = L.nnpp_params_from_reference(None, None, None, None, None, None, 0.0, 0.0, None)
    assert st == 1


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
def test_synth_deterministic(nn, kind):
    a = nn.synth(kind, 10, 5)
    b = nn.synth(kind, 10, 5)
    c = nn.synth(kind, 10, 6)
    for key in ("nodes", "bctypes", "bcvalues", "icvalues", "phase0"):
        assert np.array_equal(a[key], b[key])
    if kind != 0:
        assert not np.array_equal(a["nodes"], c["nodes"])
    N = a["N"]
    assert a["nodes"].shape == (3, N)
    # Dirichlet shell: bctypes 0 and bc values 0.1 / 0, elsewhere -1
    dirn = a["bctypes"] == 0
    assert np.all(a["bcvalues"][:4, dirn] == 0.1) and np.all(a["bcvalues"][4, dirn] == 0.0)
    assert np.all(a["bcvalues"][:, ~dirn] == -1.0)
    assert not np.any(a["phase0"][dirn])


def test_synth_lattice_block_is_the_8k_case(nn):
    inp = nn.synth(0, 20, 0)
    p = inp["params"]
    assert inp["N"] == 8000 and inp["phase0"].sum() == 1000
    assert abs(p.dx - 0.05) < 1e-15 and abs(p.delta - 3.015 * 0.05) < 1e-15
    assert abs(p.dt - 0.2 * 0.05 ** 2 / 5.3e-3) < 1e-15
    assert list(p.z) == [2.0, -1.0, -1.0, 1.0]
    assert np.allclose(list(p.D_liquid), [0.7e-3, 2.0e-3, 5.3e-3, 1.3e-3])
    assert p.k_diss == 0.05
    ic = inp["icvalues"]
    liq = (inp["phase0"] == 0) & (inp["bctypes"] == 1)
    assert np.all((ic[:4, liq] >= 0.1) & (ic[:4, liq] < 0.11))
    sol = inp["phase0"] == 1
    assert np.all(ic[0, sol] == 1.0) and np.all(ic[1:4, sol] == 0.0)


def test_synth_permutation_case_is_a_permutation(nn):
    inp = nn.synth(2, 12, 3)
    lat = nn.synth(2, 12, 3)["nodes"]
    # grid positions (before jitter) are a permutation of the lattice
    p = inp["params"]
    ijk = np.rint(inp["nodes"] / p.dx - 0.5).astype(int)
    key = ijk[0] + 12 * (ijk[1] + 12 * ijk[2])
    assert sorted(key.tolist()) == list(range(12 ** 3))
    assert not np.all(np.diff(key) > 0)
    assert np.array_equal(lat, inp["nodes"])


def test_chem_context_checks_its_arguments_before_the_device(nn):
    """nnpp_chem_create refuses kernel exponents other than 0 and a zero time step before it
    looks for a device; without one it reports NNPP_ERR_CUDA."""
    import chem_case
    g = np.load(os.path.join(GOLDEN_DIR, "chemistry.npz"))
    d2, dc, d11 = g["data2"].copy(), g["datac"].copy(), g["datac11"]
    nodes, phase, U, _, r, cell = chem_case.case_inputs(nn.synth, 0, 6, 1, d2)
    N = nodes.shape[1]
    clouds = np.tile(np.arange(N, dtype=np.int32)[:, None], (1, 2))
    lengths = np.ones(N, dtype=np.int32)
    bt = np.ones(N, dtype=np.int32)
    bv = -np.ones((11, N))
    bad = dc.copy()
    bad[1, 4] = 0.5
    with pytest.raises(nn.NNPPError) as e:
        nn.ChemImplicit(nodes, clouds, lengths, bt, bv, d2, bad, d11)
    assert e.value.status == 6
    d2z = d2.copy()
    d2z[2] = 0.0
    with pytest.raises(nn.NNPPError) as e:
        nn.ChemImplicit(nodes, clouds, lengths, bt, bv, d2z, dc, d11)
    assert e.value.status == 1
    if nn.device_count() == 0:
        with pytest.raises(nn.NNPPError) as e:
            nn.ChemImplicit(nodes, clouds, lengths, bt, bv, d2, dc, d11)
        assert e.value.status == 5
