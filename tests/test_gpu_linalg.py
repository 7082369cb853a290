"""Block sparse algebra on the GPU through the C ABI: GmlNewMatrix /
GmlMultMatVec and the vector operations against the FP64 oracle, and the
conjugate-gradient solvers (FP64, and FP32 CG inside FP64 refinement)
against the oracle's CG and its FP64 residual.

Tolerances: FP64 products within 1e-12 of the row's magnitude, FP32 within
2e-6 of it (a few units of FP32 rounding over <= 24 blocks); solves must
reach |b - A x| <= 1e-10 |b| measured by the oracle in long double."""
import ctypes

import numpy as np
import pytest

import gmlib_gb300 as G

LANES = {3: 4, 4: 4, 5: 8, 7: 8}


def random_bsr(rng, nrow, b, maxdeg=24):
    deg = rng.integers(0, maxdeg + 1, nrow)
    deg[rng.integers(0, nrow)] = maxdeg                 # at least one full row
    lin = np.zeros(nrow + 1, np.int32)
    lin[1:] = np.cumsum(deg)
    col = np.concatenate([np.sort(rng.choice(nrow, d, replace=False)) for d in deg]).astype(np.int32)
    val = rng.uniform(-1, 1, (len(col), b, b))
    return lin, col, val


def new_vector(g, arr, flt):
    a = np.ascontiguousarray(arr, np.float32 if flt == G.GmlFlt else np.float64)
    idx = G.lib.GmlNewVector(g, a.shape[0], a.shape[1], G.as_ptr(a), flt)
    assert idx > 0
    return idx


def read_vector(g, idx, nrow, b, flt):
    dt = np.float32 if flt == G.GmlFlt else np.float64
    out = G.get_data(g, G.lib.GmlxVectorData(g, idx), dt, (nrow, LANES[b]))
    return out[:, :b].astype(np.float64)


def new_matrix(g, lin, col, val, flt):
    v = np.ascontiguousarray(val, np.float32 if flt == G.GmlFlt else np.float64)
    lin_c = np.ascontiguousarray(lin, np.int32)
    col_c = np.ascontiguousarray(col, np.int32)
    IP = ctypes.POINTER(ctypes.c_int)
    idx = G.lib.GmlNewMatrix(g, len(lin) - 1, len(col), val.shape[-1], G.as_ptr(v),
                             col_c.ctypes.data_as(IP), lin_c.ctypes.data_as(IP), flt)
    assert idx > 0
    return idx


@pytest.mark.gpu
@pytest.mark.parametrize("b", [3, 4, 5, 7])
@pytest.mark.parametrize("flt", [G.GmlFlt, G.GmlDbl])
def test_multmatvec(O, gpu, b, flt):
    rng = np.random.default_rng(100 + b + 10 * flt)
    nrow = 1237                                    # ragged last slice
    lin, col, val = random_bsr(rng, nrow, b)
    x = rng.uniform(-1, 1, (nrow, b))
    if flt == G.GmlFlt:
        val = val.astype(np.float32).astype(np.float64)
        x = x.astype(np.float32).astype(np.float64)
    m = new_matrix(gpu, lin, col, val, flt)
    vx = new_vector(gpu, x, flt)
    vy = new_vector(gpu, np.zeros((nrow, b)), flt)
    assert G.lib.GmlMultMatVec(gpu, m, vy, vx) == 1           # V1 = A . V2
    y = read_vector(gpu, vy, nrow, b, flt)
    ref = O.bsr_spmv(lin, col, val, x)
    mag = O.bsr_spmv(lin, col, np.abs(val), np.abs(x)) + 1e-30
    tol = 1e-12 if flt == G.GmlDbl else 2e-6
    assert np.max(np.abs(y - ref) / mag) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("flt", [G.GmlFlt, G.GmlDbl])
def test_vector_operations(O, gpu, flt):
    rng = np.random.default_rng(7 + flt)
    nrow, b = 3001, 3
    dt = np.float32 if flt == G.GmlFlt else np.float64
    u, v, w = (rng.uniform(-1, 1, (nrow, b)).astype(dt) for _ in range(3))
    iu, iv, iw = new_vector(gpu, u, flt), new_vector(gpu, v, flt), new_vector(gpu, w, flt)
    iy = new_vector(gpu, np.zeros((nrow, b)), flt)
    assert G.lib.GmlAddVec3(gpu, iu, iv, iw, iy) == 1          # Y = U + V + W
    y = read_vector(gpu, iy, nrow, b, flt)
    exp = u.astype(np.float64) + v + w
    assert np.max(np.abs(y - exp)) <= (4e-7 if flt == G.GmlFlt else 1e-15) * 3

    mul = ctypes.c_double(-2.5)
    assert G.lib.GmlScaleVec(gpu, iy, ctypes.byref(mul)) == 1
    y2 = read_vector(gpu, iy, nrow, b, flt)
    assert np.array_equal(y2, (y.astype(dt) * dt(-2.5)).astype(np.float64))

    d = rng.uniform(-1, 1, (nrow, b * b)).astype(dt)
    idg = new_vector(gpu, d, flt)
    iz = new_vector(gpu, np.zeros((nrow, b)), flt)
    assert G.lib.GmlMultDiagMatVec(gpu, idg, iu, iz) == 1      # Z = D_line . U_line
    z = read_vector(gpu, iz, nrow, b, flt)
    zexp = np.einsum("lij,lj->li", d.reshape(nrow, b, b).astype(np.float64), u.astype(np.float64))
    assert np.max(np.abs(z - zexp)) <= (1e-6 if flt == G.GmlFlt else 1e-14)
    # the padding lane of each stored line stays zero
    raw = G.get_data(gpu, G.lib.GmlxVectorData(gpu, iz), dt, (nrow, 4))
    assert np.all(raw[:, 3] == 0)

    # scaling a vector whose stored length is not a multiple of four values
    s1 = rng.uniform(-1, 1, (nrow, 1)).astype(dt)
    i1 = new_vector(gpu, s1, flt)
    assert G.lib.GmlScaleVec(gpu, i1, ctypes.byref(mul)) == 1
    got = G.get_data(gpu, G.lib.GmlxVectorData(gpu, i1), dt, nrow)       # one value per line
    assert np.array_equal(got, s1[:, 0] * dt(-2.5))

    G.lib.GmlNewMeshData(gpu, G.GmlVertices, nrow)
    red = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 1, G.GmlFlt, b"red")
    nrm = ctypes.c_double()
    assert G.lib.GmlNormVec(gpu, iu, red, ctypes.byref(nrm)) == 1
    rows = np.sqrt((u.astype(np.float64) ** 2).sum(axis=1))
    assert nrm.value == pytest.approx(np.sqrt(rows.sum()), rel=1e-6)


def solve(g, lin, col, val, rhs, mode, tol=1e-10, maxit=5000):
    m = new_matrix(g, lin, col, val, G.GmlDbl)
    ib = new_vector(g, rhs, G.GmlDbl)
    ix = new_vector(g, np.zeros_like(rhs), G.GmlDbl)
    info = G.GmlxSolveInfo()
    rc = G.lib.GmlxSolveCG(g, m, ib, ix, mode, tol, maxit, ctypes.byref(info))
    x = read_vector(g, ix, len(lin) - 1, val.shape[-1], G.GmlDbl)
    return rc, x, info


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [G.GmlxCgFp64, G.GmlxCgMixed])
@pytest.mark.parametrize("n,split", [(6, 0), (20, 1)])
def test_cg_reaches_tolerance(O, gpu, mode, n, split):
    lin, col, val, rhs = G.cube_spd(n, split, seed=n)
    rc, x, info = solve(gpu, lin, col, val, rhs, mode)
    assert rc == 1, (rc, info.NmbIte, info.RelRes)
    rel = O.rel_residual(lin, col, val, rhs, x)
    assert rel <= 1e-10
    assert info.RelRes == pytest.approx(rel, rel=1e-3, abs=1e-13)
    xo, ito = O.cg(lin, col, val, rhs, 1e-10, 5000)
    # both residuals are below 1e-10 |b| and the smallest eigenvalue is 1
    assert np.max(np.abs(x - xo)) <= 4e-10 * np.linalg.norm(rhs)
    if mode == G.GmlxCgFp64:
        assert abs(info.NmbIte - ito) <= 2
        assert info.NmbOut == 1
    else:
        assert info.NmbOut >= 2


def spd_blocks(lin, col, b, seed):
    """An SPD system of b x b blocks on the (symmetric) sparsity of the cube
    vertex graph: off-diagonal blocks uniform in [-1, 0] with A_ji = A_ij^T,
    diagonal blocks diag(1 + sum of |entries| of the row), rhs in [-1, 1]."""
    rng = np.random.default_rng(seed)
    nrow = len(lin) - 1
    row = np.repeat(np.arange(nrow), np.diff(lin))
    key = row.astype(np.int64) * nrow + col
    tkey = col.astype(np.int64) * nrow + row
    order = np.argsort(key)
    tpos = order[np.searchsorted(key[order], tkey)]          # index of block (j, i)
    val = np.zeros((len(col), b, b))
    upper = col > row
    blk = rng.uniform(-1.0, 0.0, (int(upper.sum()), b, b))
    val[upper] = blk
    val[tpos[upper]] = np.transpose(blk, (0, 2, 1))
    diag = col == row
    absrow = np.zeros((nrow, b))
    np.add.at(absrow, row[~diag], np.abs(val[~diag]).sum(axis=2))
    val[diag] = np.eye(b)[None] * (1.0 + absrow[row[diag]])[:, :, None]
    rhs = rng.uniform(-1.0, 1.0, (nrow, b))
    return val, rhs


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [G.GmlxCgFp64, G.GmlxCgMixed])
@pytest.mark.parametrize("b", [4, 5, 7])
def test_cg_block_sizes(O, gpu, mode, b):
    """The SpMV, update and fused direction kernels of every block size
    (4- and 8-lane vector lines)."""
    lin, col, _, _ = G.cube_spd(8, 1, seed=b)
    val, rhs = spd_blocks(lin, col, b, seed=b)
    rc, x, info = solve(gpu, lin, col, val, rhs, mode)
    assert rc == 1, (rc, info.NmbIte, info.RelRes)
    rel = O.rel_residual(lin, col, val, rhs, x)
    assert rel <= 1e-10
    xo, ito = O.cg(lin, col, val, rhs, 1e-10, 5000)
    assert np.max(np.abs(x - xo)) <= 4e-10 * np.linalg.norm(rhs)
    if mode == G.GmlxCgFp64:
        assert abs(info.NmbIte - ito) <= 2


@pytest.mark.gpu
def test_cg_is_deterministic(gpu):
    lin, col, val, rhs = G.cube_spd(12, 0, seed=3)
    m = new_matrix(gpu, lin, col, val, G.GmlDbl)
    ib = new_vector(gpu, rhs, G.GmlDbl)
    ix = new_vector(gpu, np.zeros_like(rhs), G.GmlDbl)
    out = []
    for mode in (G.GmlxCgFp64, G.GmlxCgMixed, G.GmlxCgFp64, G.GmlxCgMixed):
        info = G.GmlxSolveInfo()
        assert G.lib.GmlxSolveCG(gpu, m, ib, ix, mode, 1e-10, 5000, ctypes.byref(info)) == 1
        out.append(read_vector(gpu, ix, len(lin) - 1, 3, G.GmlDbl))
    assert np.array_equal(out[0], out[2])
    assert np.array_equal(out[1], out[3])


@pytest.mark.gpu
def test_cg_breakdown_and_errors(gpu):
    """A negative definite matrix stops with the breakdown code; bad
    arguments are rejected on the host."""
    lin, col, val, rhs = G.cube_spd(4, 0, seed=1)
    rc, x, info = solve(gpu, lin, col, -val, rhs, G.GmlxCgFp64)
    assert rc == -7
    m32 = new_matrix(gpu, lin, col, val, G.GmlFlt)
    ib = new_vector(gpu, rhs, G.GmlDbl)
    ix = new_vector(gpu, np.zeros_like(rhs), G.GmlDbl)
    assert G.lib.GmlxSolveCG(gpu, m32, ib, ix, 0, 1e-10, 10, None) == -3
    assert G.lib.GmlxSolveCG(gpu, 9, ib, ix, 0, 1e-10, 10, None) == -1


@pytest.mark.gpu
def test_new_matrix_rejects_bad_csr(gpu):
    """Column indices outside the rows and decreasing row pointers are
    caught by the device repack: GmlNewMatrix returns 0 and the slot is
    free for the next matrix."""
    rng = np.random.default_rng(4)
    lin, col, val = random_bsr(rng, 200, 3, maxdeg=6)
    bad = col.copy()
    bad[len(bad) // 2] = 200
    IP = ctypes.POINTER(ctypes.c_int)
    v = np.ascontiguousarray(val)
    assert G.lib.GmlNewMatrix(gpu, 200, len(col), 3, G.as_ptr(v), bad.ctypes.data_as(IP),
                              lin.ctypes.data_as(IP), G.GmlDbl) == 0
    lin2 = lin.copy()
    lin2[100], lin2[101] = lin2[101], lin2[100]
    if lin2[100] != lin2[101]:
        assert G.lib.GmlNewMatrix(gpu, 200, len(col), 3, G.as_ptr(v), col.ctypes.data_as(IP),
                                  lin2.ctypes.data_as(IP), G.GmlDbl) == 0
    assert new_matrix(gpu, lin, col, val, G.GmlDbl) == 1
