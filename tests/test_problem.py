"""The synthetic SPD block system (GmlxCubeSpdMatrix, host code) and the
oracle's block algebra, on the CPU.  The oracle's SpMV and CG are pinned to
dense numpy linear algebra here before the GPU tests use them."""
import numpy as np
import pytest


def dense(lin, col, val):
    nv = len(lin) - 1
    b = val.shape[-1]
    A = np.zeros((b * nv, b * nv))
    for r in range(nv):
        for k in range(lin[r], lin[r + 1]):
            A[b * r:b * r + b, b * col[k]:b * col[k] + b] = val[k]
    return A


@pytest.mark.parametrize("n,split", [(1, 0), (3, 0), (4, 1), (5, 1)])
def test_spd_structure(G, n, split):
    lin, col, val, rhs = G.cube_spd(n, split, seed=11)
    m = n + 1
    edges = 3 * n * m * m + 3 * n * n * m + n ** 3
    nv = m ** 3
    assert len(lin) == nv + 1 and len(col) == 2 * edges + nv
    for r in range(nv):
        c = col[lin[r]:lin[r + 1]]
        assert np.all(np.diff(c) > 0) and r in c
    A = dense(lin, col, val)
    assert np.array_equal(A, A.T)
    off = A - np.diag(np.diag(A))
    assert np.all(off <= 0) and np.all(off >= -1)
    assert np.allclose(np.diag(A), 1.0 + np.abs(off).sum(axis=1), rtol=0, atol=1e-12)
    assert np.linalg.eigvalsh(A).min() >= 1.0 - 1e-9
    assert np.all(np.abs(rhs) <= 1.0)


def test_spd_is_deterministic(G):
    a = G.cube_spd(5, 0, seed=9)
    b = G.cube_spd(5, 0, seed=9)
    c = G.cube_spd(5, 0, seed=10)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert not np.array_equal(a[2], c[2])


def test_spd_sizes_of_the_solver_workload(G):
    import ctypes
    nl, nb = ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlxCubeSpdSizes(96, 0, ctypes.byref(nl), ctypes.byref(nb)) == 1
    assert (nl.value, nb.value) == (912673, 2 * 6276384 + 912673)


def test_oracle_spmv_and_cg_against_dense(G, O):
    lin, col, val, rhs = G.cube_spd(4, 1, seed=2)
    A = dense(lin, col, val)
    x = np.random.default_rng(0).uniform(-1, 1, rhs.shape)
    assert np.allclose(O.bsr_spmv(lin, col, val, x).ravel(), A @ x.ravel(), rtol=0, atol=1e-12)
    xs, it = O.cg(lin, col, val, rhs, 1e-12, 1000)
    assert 0 < it < 200
    exact = np.linalg.solve(A, rhs.ravel())
    assert np.max(np.abs(xs.ravel() - exact)) <= 1e-11 * np.linalg.norm(rhs)
    assert O.rel_residual(lin, col, val, rhs, xs) <= 1e-12
