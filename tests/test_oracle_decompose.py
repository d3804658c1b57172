"""The decomposition restatement (oracle/decompose.py) on CPU: every part is
the field or zero, the two parts of a field cover it, and a pulse travelling
in +y is split mostly into one side."""
import numpy as np


def test_decomposition_restatement_properties():
    from oracle import decompose, vargrid
    NX, NY, DH, DT, c = 60, 200, 5.0, 5e-4, 2000.0
    g = vargrid.VarGrid(NX, NY, 1, DH, [0], [1])
    op = vargrid.Operators(g, [4], DT, False, np.float32, var_order=False, edge=True, var_grid=False)
    y = g.y.astype(np.float64) * DH

    def fields(t):
        a = np.exp(-((y - 300.0 - c * t) / 40.0) ** 2)
        return [a.astype(np.float32), np.zeros(g.N, np.float32), (a / (2000.0 * c)).astype(np.float32)]

    cur, old = fields(DT), fields(0.0)
    parts = decompose.decompose_2d_acoustic(1, cur, old, op.Dyf, DT)
    for q in range(3):
        up, down = parts[2 * q], parts[2 * q + 1]
        F = cur[q]
        assert np.all((up == F) | (up == 0)) and np.all((down == F) | (down == 0))
        assert np.all((up == F) | (down == F))
    P = cur[0]
    m = P > 1e-3
    assert (parts[1][m] == P[m]).mean() > 0.7
    # left/right with Dxf: a field constant in x has no x-derivative, so the
    # estimate is S1 alone
    parts2 = decompose.decompose_2d_acoustic(2, cur, old, op.Dxf, DT)
    assert all(np.all((p == f) | (p == 0)) for p, f in zip(parts2, [cur[0], cur[0], cur[1], cur[1], cur[2], cur[2]]))
