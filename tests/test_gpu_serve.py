"""The request loop through the C ABI: every request gives the same result
served alone (serial mode, fresh instance per request) and in the mix
(continuous batching, resident targets, overlapping slots), including
under a memory budget that forces evictions.  Quality statistics and CG
iteration counts and residuals are compared exactly."""
import numpy as np
import pytest

import gmlib_gb300 as G

MESHES = [(3, 0, 0.3), (6, 1, 0.3), (4, 1, 0.25), (8, 0, 0.3), (5, 1, 0.2)]
SYSTEMS = [(4, 0), (6, 1)]


class Pool:
    """Registered targets; keeps the host arrays alive."""

    def __init__(self, srv):
        self.keep = []
        self.kinds = []
        for i, (n, split, jit) in enumerate(MESHES):
            crd, tet, ref = G.cube_mesh(n, split=split, jitter=jit, seed=70 + i)
            self.keep.append((crd, tet, ref))
            k = G.lib.GmlxServeAddMesh(srv, len(crd), G.as_ptr(crd), G.as_ptr(ref), len(tet),
                                       G.as_ptr(tet), 1.0 / n)
            assert k == len(self.kinds)
            self.kinds.append("mesh")
        for n, split in SYSTEMS:
            lin, col, val, rhs = G.cube_spd(n, split, seed=n)
            self.keep.append((lin, col, val, rhs))
            k = G.lib.GmlxServeAddSystem(srv, len(lin) - 1, len(col), G.as_ptr(lin), G.as_ptr(col),
                                         G.as_ptr(val), G.as_ptr(rhs))
            assert k == len(self.kinds)
            self.kinds.append("system")


def trace(kinds, n, rate, seed):
    rng = np.random.default_rng(seed)
    meshes = [i for i, k in enumerate(kinds) if k == "mesh"]
    systems = [i for i, k in enumerate(kinds) if k == "system"]
    req = (G.GmlxRequest * n)()
    t = 0.0
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        u = rng.random()
        if u < 0.5:
            req[i].kind, req[i].target = G.GmlxReqQuality, int(rng.choice(meshes))
        elif u < 0.8:
            req[i].kind, req[i].target = G.GmlxReqSmooth, int(rng.choice(meshes))
        else:
            req[i].kind, req[i].target = G.GmlxReqSolve, int(rng.choice(systems))
        req[i].arrival = t
    return req


def serve(req, mode, budget=64e9, slots=4):
    srv = G.lib.GmlxServeNew(0, budget, slots)
    assert srv
    try:
        pool = Pool(srv)
        pool.bytes = [G.lib.GmlxServeTargetBytes(srv, k) for k in range(len(pool.kinds))]
        st = G.GmlxServeStats()
        assert G.lib.GmlxServeRun(srv, req, len(req), mode, G.ctypes.byref(st)) == 1
        return pool, st
    finally:
        G.lib.GmlxServeFree(srv)


def key(r):
    q = r.qal
    if r.kind == G.GmlxReqSolve:
        return (r.status, r.NmbIte, r.RelRes)
    return (r.status, q.MinQal, q.MinIdx, q.MaxQal, q.MaxIdx, q.NmbInv, tuple(q.Hist),
            round(q.SumQal, 9))


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix():
    n = 80
    a = trace([k for k in ["mesh"] * len(MESHES) + ["system"] * len(SYSTEMS)], n, 400.0, 5)
    b = trace([k for k in ["mesh"] * len(MESHES) + ["system"] * len(SYSTEMS)], n, 400.0, 5)
    _, sa = serve(a, G.GmlxServeSerial)
    _, sb = serve(b, G.GmlxServeBatching)
    assert sa.completed == n and sb.completed == n
    for i in range(n):
        assert key(a[i]) == key(b[i]), i
        assert a[i].status == 1
        if a[i].kind == G.GmlxReqSolve:
            assert a[i].RelRes <= 1e-10
        assert b[i].finish >= b[i].start >= b[i].arrival - 1e-6
    assert sb.p50 <= sb.p99 <= sb.max
    # resident targets are loaded once each at most
    assert sb.loads <= len(MESHES) + len(SYSTEMS)
    assert sa.loads == n


@pytest.mark.gpu
def test_budget_forces_evictions_without_changing_results():
    kinds = ["mesh"] * len(MESHES) + ["system"] * len(SYSTEMS)
    n = 60
    ref = trace(kinds, n, 300.0, 9)
    p0, s0 = serve(ref, G.GmlxServeBatching)
    tight = trace(kinds, n, 300.0, 9)
    # room for two targets at a time
    budget = 2.0 * max(p0.bytes) + 1.0
    p1, s1 = serve(tight, G.GmlxServeBatching, budget=budget, slots=3)
    assert s1.completed == n and s1.evictions > 0
    assert s1.peak_bytes <= budget
    for i in range(n):
        assert key(ref[i]) == key(tight[i]), i


@pytest.mark.gpu
def test_target_larger_than_budget_fails_alone():
    kinds = ["mesh"] * len(MESHES) + ["system"] * len(SYSTEMS)
    req = trace(kinds, 20, 500.0, 3)
    probe = trace(kinds, 1, 500.0, 3)
    pool, _ = serve(probe, G.GmlxServeBatching)
    budget = sorted(pool.bytes)[2] + 1.0          # the three smallest targets fit
    _, st = serve(req, G.GmlxServeBatching, budget=budget, slots=2)
    fits = [pool.bytes[req[i].target] <= budget for i in range(20)]
    assert 0 < sum(fits) < 20
    assert st.completed == sum(fits)
    for i in range(20):
        assert req[i].status == (1 if fits[i] else 0), i
