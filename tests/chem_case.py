"""Inputs of the ten-species residual cases (shared by tests/golden/make_golden.py, which
runs the reference's utils::Residuals on them, and the GPU test): a synthetic workload's
lattice and phases rescaled to the node spacing of the reference's data files, and seeded
concentrations and potentials at two time levels in the ranges where every reaction term of
utils.h is active."""
import numpy as np

CASES = [(0, 12, 3), (1, 12, 3)]
VOLN1REL = 0.3


def case_inputs(synth, kind, n, seed, data2):
    """(nodes (3, N), phase (N,), Un1 (11, N), Un (11, N), r, cell) of one case; synth is
    nnpp_gb300.synth or oracle.synth (the same bits)."""
    inp = synth(kind, n, seed)
    dx = float(data2[3])
    nodes = np.ascontiguousarray(inp["nodes"] * (dx / inp["params"].dx))
    phase = np.ascontiguousarray(inp["phase0"], dtype=np.int32)
    N = nodes.shape[1]
    rng = np.random.default_rng(1000 * kind + seed)
    Un = np.empty((11, N))
    Un[:10] = 10.0 ** rng.uniform(-5.0, -2.0, (10, N))   # concentrations / CSolid
    Un[10] = 0.01 * rng.standard_normal(N)                # potential (V)
    Un1 = Un * (1.0 + 1e-3 * rng.standard_normal((11, N)))
    r = float(data2[6]) * (1.0 + 1e-5)
    return nodes, phase, Un1, Un, r, 10.0 * dx


def reactive_data2(data2):
    """The reference's data2 with rate and solubility constants chosen so that the reaction
    terms reach the transport terms' size and each max(., 0) is active on about half of the
    nodes (thresholds at the median products of case_inputs' log-uniform concentrations,
    10^-3.5 each), and a cathodic H+ source of the same size: a test of the reaction terms,
    which the physical constants leave ~1e-12 of the residual."""
    d2 = np.array(data2, dtype=np.float64).copy()
    lcs = np.log10(d2[7])  # CSolid
    # median log10 products: MgOH2 U1 U3^2, MgCO3 / MgHCO3 U1 U5, MgPO4 U1^3 U6^2, CaCO3 U5 U8,
    # Ca5OHPO4 U3 U8^5 U7^3, and the water / HCO3 / HPO4 equilibria's two-factor products
    med = {14: -10.5, 15: -7.0, 16: -7.0, 17: -17.5, 18: -7.0, 19: -31.5, 20: -7.0, 21: -7.0, 22: -7.0}
    for i, m in med.items():
        d2[i] = -(m + lcs)
    d2[16] += 0.3  # MgHCO3's threshold apart from MgCO3's
    # k_b: rate times the largest product (concentrations up to 10^-2) ~1, the size of the
    # transport terms
    kb = {29: 6.0, 31: 4.0, 33: 4.0, 35: 10.0, 37: 4.0, 39: 18.0, 41: 4.0, 43: 4.0, 45: 4.0}
    for i, m in kb.items():
        d2[i] = 10.0 ** m
    d2[46] = -5e7   # JHp
    d2[27] = 0.05   # alphaC
    return d2
