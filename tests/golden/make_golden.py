"""Generate the golden fixtures of tests/golden/ from the reference's own code.

Runs the reference's build_clouds_hash (grid.h:43-204), utils::Residuals (utils.h:29-842)
and utils::NewtonMatrices' K11 (utils.h:1794-1848), compiled from the reference's sources
by oracle/build_oracle.py, on the synthetic workloads of nnpp_synth_fill, and stores:
  clouds.json     SHA-256 of the reference's neighbour lists (lengths and padded rows) for
                  small cases of every geometry kind and for the full 8k, 512k and 2M
                  workloads, with the max cloud length and the bond count
  residuals.npz   F1..F4, F11 of the reference for a seeded state on small cases
  k11.json        SHA-256 and sums of the reference's K11 entries on a small case
  synth.json      SHA-256 of the generated node coordinates (cross-platform determinism)
  params.json     the reference's control vectors of data/NNPP.data2, .datac1-4, .datac11
  implant.json    SHA-256 of the point counts of the reference's kd-tree implant query for
                  seeded implant point clouds
  chemistry.npz   F1..F11 of the reference's complete residual (ten species, reactions) with
                  the control vectors of its data files, on the cases of tests/chem_case.py
Needs the reference's sources (REFERENCE_ROOT); run:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
# the reference checkout: NNPP_REFERENCE_ROOT, else "reference" beside this repository
REFERENCE_ROOT = os.environ.get("NNPP_REFERENCE_ROOT",
                                os.path.normpath(os.path.join(ROOT, "..", "reference")))

SMALL = [(0, 20, 11), (1, 16, 11), (2, 14, 11), (3, 20, 11), (4, 15, 11)]
FULL = [("lattice_block_20", 0, 20, 0), ("jittered_sphere_80", 1, 80, 1),
        ("screw_permuted_126", 2, 126, 1)]
RESID = [(0, 12, 3), (1, 12, 3), (2, 12, 3)]


def clouds_digest(lengths, ptr, cols):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(lengths, dtype=np.int32).tobytes())
    h.update(np.ascontiguousarray(cols, dtype=np.int32).tobytes())
    return h.hexdigest()


def nodes_digest(nodes):
    return hashlib.sha256(np.ascontiguousarray(nodes, dtype=np.float64).tobytes()).hexdigest()


def residual_state(N, seed):
    rng = np.random.default_rng(seed)
    c = 0.05 + rng.random((4, N))
    phi = rng.standard_normal(N) * 0.3
    return c, phi


# implant point clouds (oracle.synth_implant_points) on the nodes of synthetic workloads
IMPLANT = [(0, 20, 0, "sphere"), (1, 24, 3, "shell"), (1, 16, 5, "sphere")]


def implant_fixtures():
    """Point counts of the reference's kd-tree implant query (kd_tree_interface.h:156-252,
    as main.cpp:316-325 calls it with r = 3 * 0.4 dx (1 + 1e-5)) -> implant.json."""
    import ctypes as C
    import oracle as O
    L = O.load_reference()
    out = {}
    for kind, n, seed, shape in IMPLANT:
        inp = O.synth(kind, n, seed)
        nodes = np.ascontiguousarray(inp["nodes"])
        pts = O.synth_implant_points(n, seed, shape)
        r = 3 * 0.4 * inp["params"].dx * (1 + 1e-5)
        N = nodes.shape[1]
        counts = np.empty(N, dtype=np.int32)
        st = L.ref_implant_counts(N, nodes.ctypes.data_as(C.POINTER(C.c_double)), pts.shape[1],
                                  pts.ctypes.data_as(C.POINTER(C.c_double)), r, 1024,
                                  counts.ctypes.data_as(C.POINTER(C.c_int)))
        if st != 0:
            raise SystemExit("reference implant query failed")
        key = "kind%d_n%d_seed%d_%s" % (kind, n, seed, shape)
        out[key] = {"kind": kind, "n_side": n, "seed": seed, "shape": shape, "r": r, "N": int(N),
                    "M": int(pts.shape[1]), "points_sha256": nodes_digest(pts),
                    "counts_sha256": hashlib.sha256(counts.tobytes()).hexdigest(),
                    "solid": int((counts > 0).sum()), "sum": int(counts.sum())}
        print(key, out[key], flush=True)
    with open(os.path.join(HERE, "implant.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


def read_control(name):
    """A whitespace-separated control vector of the reference's data directory."""
    with open(os.path.join(REFERENCE_ROOT, "data", name)) as f:
        return np.array([float(x) for x in f.read().split()])


def chemistry_fixtures():
    """chemistry.npz: the reference's complete residual (ten species, their reactions, the
    potential; utils.h:29-842) with the control vectors of its data files (NNPP.data2,
    .datac1-10, .datac11) on the cases of tests/chem_case.py, and those vectors."""
    import chem_case
    import oracle as O
    if O.load_reference() is None:
        raise SystemExit("reference sources not found at %s" % REFERENCE_ROOT)
    d2 = read_control("NNPP.data2")
    dc = np.stack([read_control("NNPP.datac%d" % k) for k in range(1, 11)])
    d11 = read_control("NNPP.datac11")
    assert d2.shape == (51,) and dc.shape == (10, 7) and d11.shape == (4,)
    arrays = {"data2": d2, "datac": dc, "datac11": d11}
    d2r = chem_case.reactive_data2(d2)
    d2z = d2r.copy()
    d2z[[29, 31, 33, 35, 37, 39, 41, 43, 45, 46]] = 0.0  # no reaction, no H+ source
    for kind, n, seed in chem_case.CASES:
        nodes, phase, Un1, Un, r, cell = chem_case.case_inputs(O.synth, kind, n, seed, d2)
        lo, po, co, ml = O.ref_build_clouds_hash(1024, r, cell, cell, cell, nodes)
        key = "kind%d_n%d_seed%d" % (kind, n, seed)
        F = O.ref_residuals_full(nodes, po, co, Un1, Un, phase, chem_case.VOLN1REL, d2, dc, d11)
        Fr = O.ref_residuals_full(nodes, po, co, Un1, Un, phase, chem_case.VOLN1REL, d2r, dc, d11)
        Fz = O.ref_residuals_full(nodes, po, co, Un1, Un, phase, chem_case.VOLN1REL, d2z, dc, d11)
        arrays[key + "_F"] = F
        arrays[key + "_Freactive"] = Fr
        print(key, "N", nodes.shape[1], "max|F| per field", np.abs(F).max(axis=1), flush=True)
        print("   reactive: max|F|", np.abs(Fr).max(axis=1), "max|R|", np.abs(Fr - Fz).max(axis=1), flush=True)
    np.savez_compressed(os.path.join(HERE, "chemistry.npz"), **arrays)


def main():
    if "--only-implant" in sys.argv:
        implant_fixtures()
        return
    if "--only-chemistry" in sys.argv:
        chemistry_fixtures()
        return
    from conftest import load_package
    import oracle as O
    nn = load_package()
    if O.load_reference() is None:
        raise SystemExit("reference sources not found at %s" % REFERENCE_ROOT)
    clouds = {}
    synth = {}
    for kind, n, seed in SMALL:
        inp = nn.synth(kind, n, seed)
        p = inp["params"]
        lo, po, co, ml = O.ref_build_clouds_hash(1024, p.delta * (1 + 1e-5), p.dx * 10, p.dy * 10,
                                                 p.dz * 10, inp["nodes"])
        key = "kind%d_n%d_seed%d" % (kind, n, seed)
        clouds[key] = {"sha256": clouds_digest(lo, po, co), "max_len": int(ml), "nnz": int(po[-1])}
        synth[key] = nodes_digest(inp["nodes"])
        print(key, clouds[key], flush=True)
    for name, kind, n, seed in FULL:
        inp = nn.synth(kind, n, seed)
        p = inp["params"]
        lo, po, co, ml = O.ref_build_clouds_hash(1024, p.delta * (1 + 1e-5), p.dx * 10, p.dy * 10,
                                                 p.dz * 10, inp["nodes"])
        clouds[name] = {"kind": kind, "n_side": n, "seed": seed, "sha256": clouds_digest(lo, po, co),
                        "max_len": int(ml), "nnz": int(po[-1]), "N": int(inp["N"])}
        synth[name] = nodes_digest(inp["nodes"])
        print(name, clouds[name], flush=True)
    with open(os.path.join(HERE, "clouds.json"), "w") as f:
        json.dump(clouds, f, indent=1, sort_keys=True)
    with open(os.path.join(HERE, "synth.json"), "w") as f:
        json.dump(synth, f, indent=1, sort_keys=True)

    arrays = {}
    for kind, n, seed in RESID:
        inp = nn.synth(kind, n, seed)
        p = inp["params"].copy()
        p.k_diss = 0.0
        p.vol_red = 0.5
        N = inp["N"]
        lo, po, co, ml = O.ref_build_clouds_hash(1024, p.delta * (1 + 1e-5), p.dx * 10, p.dy * 10,
                                                 p.dz * 10, inp["nodes"])
        c, phi = residual_state(N, 100 + kind)
        F = O.ref_residuals(p, inp["nodes"], po, co, c, phi, inp["phase0"], inp["bctypes"],
                            inp["bcvalues"], voln1rel=0.25)
        key = "kind%d_n%d_seed%d" % (kind, n, seed)
        arrays[key + "_F"] = np.concatenate([F[:4], F[10:11]])
    np.savez_compressed(os.path.join(HERE, "residuals.npz"), **arrays)

    kind, n, seed = RESID[1]
    inp = nn.synth(kind, n, seed)
    p = inp["params"]
    lo, po, co, ml = O.ref_build_clouds_hash(1024, p.delta * (1 + 1e-5), p.dx * 10, p.dy * 10,
                                             p.dz * 10, inp["nodes"])
    c, phi = residual_state(inp["N"], 100 + kind)
    ri, ci, val = O.ref_k11(p, inp["nodes"], po, co, c, phi, inp["phase0"], inp["bctypes"],
                            inp["bcvalues"])
    order = np.lexsort((ci, ri))
    h = hashlib.sha256()
    h.update(ri[order].astype(np.int32).tobytes())
    h.update(ci[order].astype(np.int32).tobytes())
    h.update(val[order].astype(np.float64).tobytes())
    k11 = {"case": "kind%d_n%d_seed%d" % (kind, n, seed), "nnz": int(len(val)),
           "sha256": h.hexdigest(), "sum": float(val.sum()), "abs_sum": float(np.abs(val).sum())}
    with open(os.path.join(HERE, "k11.json"), "w") as f:
        json.dump(k11, f, indent=1)

    data = os.path.join(REFERENCE_ROOT, "data")
    params = {}
    for name, size in [("NNPP.data2", 51), ("NNPP.datac1", 7), ("NNPP.datac2", 7),
                       ("NNPP.datac3", 7), ("NNPP.datac4", 7), ("NNPP.datac11", 4)]:
        with open(os.path.join(data, name)) as f:
            vals = [float(t) for t in f.read().split()][:size]
        params[name] = vals
    with open(os.path.join(HERE, "params.json"), "w") as f:
        json.dump(params, f, indent=1)
    implant_fixtures()
    print("fixtures written", flush=True)


if __name__ == "__main__":
    main()
