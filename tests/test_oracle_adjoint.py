"""The oracle's FP64 adjoint of the explicit step against central finite differences
(h = 1e-5 relative), on a small jittered-sphere case with the sigmoid dissolution switch."""
import numpy as np


def _params(inp, scale_D=1.0, k=0.05):
    p = inp["params"].copy()
    p.switch_width = 0.01
    p.k_diss = k
    for s in range(4):
        p.D_liquid[s] *= scale_D
        p.D_solid[s] *= scale_D
    return p


def _run(orc, inp, p, n_steps, se):
    o = orc.Oracle(p, inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"], inp["phase0"])
    o.build_neighbours()
    o.set_solver(1e-14)
    return o, orc.oracle_forward_record(o, n_steps, se)


def test_oracle_adjoint_matches_central_differences(nn, orc):
    inp = nn.synth(1, 12, 5)
    n_steps, se = 60, 20
    _, target = _run(orc, inp, _params(inp, 1.2, 0.06), n_steps, se)
    base = _params(inp)
    o, curve = _run(orc, inp, base, n_steps, se)
    gD, gk = orc.oracle_backward(o, 2.0 * (curve - target))

    def loss(p):
        return float(((_run(orc, inp, p, n_steps, se)[1] - target) ** 2).sum())

    h = 1e-5
    # the potential solve's 1e-14 tolerance sets the finite-difference noise floor: species 0
    # and the rate constant drive the loss directly and match to ~1e-8, species 1-3 act only
    # through the potential and through migration (gradients 100-1000x smaller)
    tol = (1e-7, 5e-5, 5e-5, 5e-5)
    for k in range(4):
        pp, pm = base.copy(), base.copy()
        v = base.D_liquid[k]
        for q, f in ((pp, 1 + h), (pm, 1 - h)):
            q.D_liquid[k] = v * f
            q.D_solid[k] = base.D_solid[k] * f
        fd = (loss(pp) - loss(pm)) / (2 * h * v)
        assert abs(gD[k] - fd) <= tol[k] * abs(fd), (k, gD[k], fd)
    pp, pm = base.copy(), base.copy()
    pp.k_diss = base.k_diss * (1 + h)
    pm.k_diss = base.k_diss * (1 - h)
    fd = (loss(pp) - loss(pm)) / (2 * h * base.k_diss)
    assert abs(gk - fd) <= 1e-9 * abs(fd), (gk, fd)
