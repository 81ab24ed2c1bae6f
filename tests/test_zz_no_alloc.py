"""The allocation-free neighbour build (nnpp_build_clouds_hash_noalloc).

It serves callers that cannot call cudaMalloc -- code whose device memory is owned by a
host framework, real-time loops that must not reach the allocator, applications at their
memory cap.  They pass their own device buffers, and every temporary lives in one fixed
device array of the library.  This test calls it through the C ABI with buffers the test
owns, twice in a row on different inputs (so the second call runs on the scratch the
first one left behind), and checks each result against the allocating entry point
nnpp_build_clouds_hash in the same (canonical) order, bit for bit.  It also checks that
inputs above the fixed maximum are refused.  This file sorts last so that a run stopping
at its first failure has run every other test before it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _expected(nn, inp, max_node_no, cell=10.0):
    p = inp["params"]
    r = p.delta * (1 + 1e-5)
    return nn.build_clouds_hash(max_node_no, r, p.dx * cell, p.dy * cell, p.dz * cell,
                                inp["nodes"], order_mode=nn.ORDER_CANONICAL)


def _noalloc(nn, torch, inp, max_node_no, cell=10.0):
    p = inp["params"]
    r = p.delta * (1 + 1e-5)
    N = inp["N"]
    d_nodes = torch.from_numpy(np.ascontiguousarray(inp["nodes"])).cuda()
    d_clouds = torch.zeros(max_node_no * N, dtype=torch.int32, device="cuda")
    d_len = torch.zeros(N, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ml = nn.build_clouds_hash_noalloc(max_node_no, r, p.dx * cell, p.dy * cell, p.dz * cell, N,
                                      d_nodes.data_ptr(), d_clouds.data_ptr(), d_len.data_ptr())
    torch.cuda.synchronize()
    clouds = d_clouds.cpu().numpy().reshape(max_node_no, N).T
    return clouds, d_len.cpu().numpy(), ml


def test_noalloc_build_matches_allocating_build_twice(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    max_node_no = 256
    for kind, n, seed in [(1, 20, 3), (2, 18, 4)]:
        inp = nn.synth(kind, n, seed)
        c_ref, l_ref, ml_ref = _expected(nn, inp, max_node_no)
        c, l, ml = _noalloc(nn, torch, inp, max_node_no)
        assert ml == ml_ref
        assert np.array_equal(l, l_ref)
        assert np.array_equal(c, c_ref)


def test_noalloc_small_cells_match_allocating_build_and_oracle_sets(nn, orc):
    """Cells of one lattice spacing give a hash grid of more than 1024 cells, so the
    two-level scan of the cell counts (block sums) runs; the lists also equal the oracle's
    reference-order lists as sets."""
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    max_node_no = 256
    inp = nn.synth(1, 20, 7)
    N = inp["N"]
    c_ref, l_ref, ml_ref = _expected(nn, inp, max_node_no, cell=1.0)
    for _ in range(2):
        c, l, ml = _noalloc(nn, torch, inp, max_node_no, cell=1.0)
        assert ml == ml_ref and np.array_equal(l, l_ref) and np.array_equal(c, c_ref)
    o = orc.Oracle.from_synth(inp)
    assert o.build_neighbours(max_node_no) == ml
    lo, po, co = o.clouds()
    assert np.array_equal(lo, l)
    for i in range(N):
        assert c[i, 0] == i
        assert np.array_equal(np.sort(c[i, 1:l[i]]), np.sort(co[po[i] + 1:po[i + 1]]))


def test_noalloc_rejects_a_hash_grid_beyond_its_maximum(nn):
    """8,000 nodes with cells of a quarter spacing: an 80^3 grid (512,000 cells) is above
    the 262,144-cell scratch maximum and is refused before any kernel writes the cell
    arrays."""
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    inp = nn.synth(1, 20, 7)
    with pytest.raises(nn.NNPPError) as ei:
        _noalloc(nn, torch, inp, 256, cell=0.25)
    assert ei.value.status == 1
    assert "cells" in str(ei.value)
    # the scratch is still usable afterwards
    c_ref, l_ref, _ = _expected(nn, inp, 256)
    c, l, _ = _noalloc(nn, torch, inp, 256)
    assert np.array_equal(c, c_ref) and np.array_equal(l, l_ref)


def test_hash_grid_overflow_is_refused_by_both_builds(nn):
    """Two nodes a unit apart with cells of 1e-4: 1e12 cells, beyond the int hash of
    grid.h:81-85.  Both builds refuse it instead of indexing with wrapped hashes."""
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    nodes = np.array([[0.0, 1.0], [0.0, 1.0], [0.0, 1.0]])
    with pytest.raises(nn.NNPPError) as ei:
        nn.build_clouds_hash(8, 1e-3, 1e-4, 1e-4, 1e-4, nodes)
    assert ei.value.status == 1
    d_nodes = torch.from_numpy(np.ascontiguousarray(nodes)).cuda()
    d_clouds = torch.zeros(16, dtype=torch.int32, device="cuda")
    d_len = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(nn.NNPPError) as ei:
        nn.build_clouds_hash_noalloc(8, 1e-3, 1e-4, 1e-4, 1e-4, 2, d_nodes.data_ptr(),
                                     d_clouds.data_ptr(), d_len.data_ptr())
    assert ei.value.status == 1


def test_noalloc_rejects_sizes_beyond_its_maximum(nn):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(nn.NNPPError) as ei:
        nn.build_clouds_hash_noalloc(128, 0.1, 1.0, 1.0, 1.0, 262145, buf.data_ptr(),
                                     buf.data_ptr(), buf.data_ptr())
    assert ei.value.status == 1
    assert "262144" in str(ei.value)
