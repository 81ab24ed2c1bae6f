"""Boundary conditions of the complete model's cases (ten species and the potential) on a
synthetic workload: the synthetic workload's Dirichlet nodes hold the four modelled species
and the potential; species 5-10 take their own values on the same nodes (field 5 on every
other one only), so that every field has Dirichlet rows and free rows."""
import numpy as np


def bc11(inp, U, csolid):
    """(bctypes (N,), bcvalues (11, N)) from the synthetic case inp and the state U (11, N):
    the synthetic rows for fields 1-4 and 11, for fields 5-10 the state's value at the
    Dirichlet nodes (in the data files' units, times CSolid)."""
    bt = np.asarray(inp["bctypes"], dtype=np.int32)
    b5 = np.asarray(inp["bcvalues"], dtype=np.float64)
    N = bt.size
    bv = -np.ones((11, N))
    bv[:4] = b5[:4]
    bv[10] = b5[4]
    on = (bt == 0) & (b5[0] != -1)
    for k in range(4, 10):
        m = on.copy()
        if k == 4:
            m[::2] = False
        bv[k, m] = U[k, m] * csolid
    return bt, bv
