"""The C++ job-file driver (nnpp_run): synthetic jobs written in the reference's input layout
read back exactly (CPU), and a run of the driver on such a job matches the FP64 oracle (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR

DRIVER = os.path.join(PKG_DIR, "nnpp_run")


def _driver():
    if not os.path.exists(DRIVER):
        pytest.fail("nnpp_run has not been built (build.py builds it with the library)")
    return DRIVER


def _load(path, dtype=float):
    return np.loadtxt(path, dtype=dtype)


def _write(job, kind, n, seed, steps):
    r = subprocess.run([_driver(), "--write-synth", str(kind), str(n), str(seed), job,
                        "--steps", str(steps)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def test_write_synth_reads_back_exactly(nn, tmp_path):
    job = str(tmp_path / "SYN")
    _write(job, 1, 8, 3, 40)
    inp = nn.synth(1, 8, 3)
    N = inp["N"]
    d1 = _load(job + ".data1", int)
    assert d1[0] == N and d1[1] == 40 and d1[3] == 0
    assert d1[2] == int((inp["bctypes"] == 0).sum())
    nodes = _load(job + ".nodes")
    assert nodes.shape == (N, 3)
    assert np.array_equal(nodes, np.asarray(inp["nodes"]).reshape(3, N).T)
    assert np.array_equal(_load(job + ".bctypes", int), inp["bctypes"])
    assert np.array_equal(_load(job + ".phase0", int), inp["phase0"])
    bcv = np.asarray(inp["bcvalues"]).reshape(5, N)
    icv = np.asarray(inp["icvalues"]).reshape(5, N)
    for f in range(1, 12):
        src = f - 1 if f <= 4 else (4 if f == 11 else None)
        b = _load(job + ".bcvalues%d" % f)
        i = _load(job + ".icvalues%d" % f)
        if src is None:
            assert np.all(b == -1) and np.all(i == 0)
        else:
            assert np.array_equal(b, bcv[src]) and np.array_equal(i, icv[src])
    # the parameter files give back the same parameters through the reference-vector entry point
    d2 = _load(job + ".data2")
    dc = [_load(job + ".datac%d" % c) for c in range(1, 5)]
    d11 = _load(job + ".datac11")
    p = nn.params_from_reference(d2, np.array(dc), d11)
    q = inp["params"]
    for name in ("dt", "dx", "dy", "dz", "delta", "CSolid", "CSat", "F", "R", "T", "vol_red",
                 "sigma", "s_phi", "K_phi"):
        assert getattr(p, name) == getattr(q, name), name
    for name in ("z", "D_solid", "D_liquid", "s1", "s2", "K1", "K2"):
        assert list(getattr(p, name)) == list(getattr(q, name)), name


def test_usage_errors():
    r = subprocess.run([_driver()], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "usage" in r.stderr
    r = subprocess.run([_driver(), "--write-synth", "9", "8", "1", "/nonexistent/x"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    r = subprocess.run([_driver(), "-x", "/nonexistent/x", "--model", "seven"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "usage" in r.stderr and "--model" in r.stderr


@pytest.mark.gpu
def test_driver_run_matches_oracle(nn, orc, tmp_path):
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    job = str(tmp_path / "SYN")
    steps = 40
    _write(job, 1, 12, 7, steps)
    r = subprocess.run([_driver(), "-fp64", job, "--precision", "fp64", "--tol", "1e-12"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    inp = nn.synth(1, 12, 7)
    p = inp["params"].copy()
    p.k_diss = 0.05
    p.switch_width = 0.0
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    o.set_solver(1e-13)
    o.forward(steps)
    c, phi, ph, _ = o.state()
    out = np.loadtxt(job + "-fp64-%d.output.csv" % steps, delimiter=",", skiprows=1)
    with open(job + "-fp64-%d.output.csv" % steps) as f:
        assert f.readline().strip().split(",")[:4] == ["X", "Y", "Z", "Mg++"]
    N = inp["N"]
    assert out.shape == (N, 15)
    assert np.array_equal(out[:, 14].astype(int), ph)
    for k in range(4):
        assert np.linalg.norm(out[:, 3 + k] - c[k]) <= 1e-10 * np.linalg.norm(c[k])
    assert np.linalg.norm(out[:, 13] - phi) <= 1e-9 * np.linalg.norm(phi)
    vol = [float(x.strip().rstrip(",")) for x in open(job + "-fp64.volume") if x.strip()]
    assert len(vol) == steps // 8
    assert len(open(job + "-fp64.energy").read().split()) == steps // 8


@pytest.mark.gpu
def test_driver_restart_continues_the_run(nn, tmp_path):
    """main.cpp:507-542: a run restarted from its own step-8 output CSV (state read back by
    column name) ends at step 16 where the uninterrupted run does (to the solver tolerance:
    the file holds 16 significant digits and the restart has no warm-start history)."""
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    import shutil
    job = str(tmp_path / "SYN")
    _write(job, 1, 12, 7, 16)
    common = ["--precision", "fp64", "--tol", "1e-12", "--every", "8"]
    r = subprocess.run([_driver(), "-a", job] + common, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    shutil.copy(job + "-a-8.output.csv", job + "-b-8.output.csv")
    r = subprocess.run([_driver(), "-b", job, "8"] + common, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Restart from" in r.stdout
    a = np.loadtxt(job + "-a-16.output.csv", delimiter=",", skiprows=1)
    b = np.loadtxt(job + "-b-16.output.csv", delimiter=",", skiprows=1)
    assert np.array_equal(a[:, :3], b[:, :3]) and np.array_equal(a[:, 14], b[:, 14])
    assert np.array_equal(a[:, 7:13], b[:, 7:13])  # the passive columns carried through
    for col in list(range(3, 7)) + [13]:
        assert np.linalg.norm(a[:, col] - b[:, col]) <= 1e-9 * np.linalg.norm(a[:, col]), col
    assert len([x for x in open(job + "-b.volume") if x.strip()]) == 1


@pytest.mark.gpu
def test_driver_implant_point_cloud(nn, orc, tmp_path):
    """BunnyConditions = 1 (main.cpp:236-240, 316-325, 422-457): with data1[3] implant points
    in <job>.bunnyNodes the nodes within 3 * 0.4 dx (1 + 1e-5) of one start solid (Mg2+ 1),
    the others liquid; the driver's phases equal the oracle's kd-tree restatement."""
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    job = str(tmp_path / "SYN")
    _write(job, 1, 16, 5, 8)
    pts = orc.synth_implant_points(16, 5, "sphere")
    d1 = _load(job + ".data1", int)
    d1[3] = pts.shape[1]
    np.savetxt(job + ".data1", d1, fmt="%d")
    np.savetxt(job + ".bunnyNodes", pts.T, fmt="%.17g")
    r = subprocess.run([_driver(), "-i", job, "--precision", "fp64", "--every", "8"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Building bunnyNodes took" in r.stdout
    inp = orc.synth(1, 16, 5)
    rad = 3 * 0.4 * inp["params"].dx * (1 + 1e-5)
    mask = (orc.implant_counts(inp["nodes"], pts, rad) > 0).astype(int)
    out = np.loadtxt(job + "-i-8.output.csv", delimiter=",", skiprows=1)
    assert np.array_equal(out[:, 14].astype(int), mask)
    # solid nodes start at Mg2+ 1 and lose a few percent in 8 steps; the implant reaches into
    # the Dirichlet shell, whose nodes hold their boundary value (main.cpp:676-712)
    dirichlet = (inp["bctypes"] == 0) & (inp["bcvalues"][0] != -1)
    inner = (mask == 1) & ~dirichlet
    assert inner.sum() > 0 and np.all(out[inner, 3] > 0.9)
    assert np.all(out[(mask == 1) & dirichlet, 3] == inp["bcvalues"][0][(mask == 1) & dirichlet])


@pytest.mark.gpu
def test_driver_full_model_matches_oracle(nn, orc, tmp_path):
    """--model full: the reference's complete model with its implicit time loop from the job
    files (nnpp_chem_*), three steps against the oracle's restatement on the same files."""
    if nn.device_count() < 1:
        pytest.skip("no CUDA device")
    job = str(tmp_path / "SYN")
    steps = 3
    _write(job, 1, 10, 5, steps)
    r = subprocess.run([_driver(), "-full", job, "--model", "full", "--every", "3"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "complete model" in r.stdout
    N = int(_load(job + ".data1", int)[0])
    d2 = _load(job + ".data2")
    dc = np.array([_load(job + ".datac%d" % c) for c in range(1, 11)])
    d11 = _load(job + ".datac11")
    nodes = np.ascontiguousarray(_load(job + ".nodes").T)
    bt = _load(job + ".bctypes", int).astype(np.int32)
    bv = np.array([_load(job + ".bcvalues%d" % f) for f in range(1, 12)])
    U = np.array([_load(job + ".icvalues%d" % f) for f in range(1, 12)])
    ph = _load(job + ".phase0", int).astype(np.int32)
    p = nn.params_from_reference(d2, dc[:4], d11)
    o = orc.Oracle(p, nodes, bt, bv[[0, 1, 2, 3, 10]], U[[0, 1, 2, 3, 10]], ph)
    o.build_neighbours(1024, d2[6] * (1 + 1e-5), (d2[3] * 10, d2[4] * 10, d2[5] * 10))
    for _ in range(steps):
        U, ph, _, _ = o.chem_implicit_step(U, ph, bt, bv, 0.0, d2, dc, d11)
    out = np.loadtxt(job + "-full-%d.output.csv" % steps, delimiter=",", skiprows=1)
    assert out.shape == (N, 15)
    assert np.array_equal(out[:, 14].astype(int), ph)
    for f in range(11):
        col = 3 + f
        scale = np.linalg.norm(U[f]) or 1.0
        assert np.linalg.norm(out[:, col] - U[f]) <= 1e-12 * scale + 1e-300, f
