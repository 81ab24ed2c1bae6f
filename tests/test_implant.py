"""The implant mask from a point cloud (nnpp_implant_mask; main.cpp:316-325, 422-457 with
kd_tree_interface.h:156-252).

CPU: the oracle's restatement (every point against every node: box node +- r, Euclidean
distance <= r) reproduces the point counts of the reference's own kd-tree query, pinned by
the digests of tests/golden/implant.json (made by tests/golden/make_golden.py from the
reference's build_clouds).  GPU: the library's counts and phases equal the oracle's, bit for
bit, and a count above max_node_no is the reference's capacity error."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR


def _cases():
    with open(os.path.join(GOLDEN_DIR, "implant.json")) as f:
        return sorted(json.load(f).items())


def _inputs(orc, g):
    inp = orc.synth(g["kind"], g["n_side"], g["seed"])
    pts = orc.synth_implant_points(g["n_side"], g["seed"], g["shape"])
    return inp, pts


@pytest.mark.parametrize("key,g", _cases())
def test_oracle_implant_counts_match_reference(orc, key, g):
    inp, pts = _inputs(orc, g)
    assert hashlib.sha256(np.ascontiguousarray(pts).tobytes()).hexdigest() == g["points_sha256"]
    counts = orc.implant_counts(inp["nodes"], pts, g["r"])
    assert hashlib.sha256(counts.astype(np.int32).tobytes()).hexdigest() == g["counts_sha256"], key
    assert int((counts > 0).sum()) == g["solid"]


@pytest.mark.gpu
@pytest.mark.parametrize("key,g", _cases())
def test_gpu_implant_mask_bit_exact(nn, orc, key, g):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    inp, pts = _inputs(orc, g)
    counts, phase = nn.implant_mask(inp["nodes"], pts, g["r"])
    ref = orc.implant_counts(inp["nodes"], pts, g["r"])
    assert np.array_equal(counts, ref), key
    assert np.array_equal(phase, (ref > 0).astype(np.int32))
    assert hashlib.sha256(counts.astype(np.int32).tobytes()).hexdigest() == g["counts_sha256"]


@pytest.mark.gpu
def test_gpu_implant_mask_capacity_and_empty_cloud(nn, orc):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    inp = orc.synth(0, 20, 0)
    pts = orc.synth_implant_points(20, 0, "sphere")
    r = 3 * 0.4 * inp["params"].dx * (1 + 1e-5)
    with pytest.raises(nn.NNPPError) as e:
        nn.implant_mask(inp["nodes"], pts, r, max_node_no=16)
    assert e.value.status == 2  # NNPP_ERR_CAPACITY
    counts, phase = nn.implant_mask(inp["nodes"], np.zeros((3, 0)), r)
    assert not counts.any() and not phase.any()
