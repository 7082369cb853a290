"""The oracle against the golden fixtures made from the reference's own
kernel bodies, and against hand-derived known answers."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["kuhn_n5.npz", "reflected_n6.npz"]


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


@pytest.mark.parametrize("case", CASES)
def test_quality_matches_reference_bodies(O, case):
    g = load(case)
    q = O.quality_ref(g["crd"], g["tet"])
    # the fixture is the reference body evaluated in FP32 on the CPU
    assert np.max(np.abs(q - g["quality"])) <= 1e-6 * np.max(np.abs(q))


@pytest.mark.parametrize("case", CASES)
def test_scatter_gather_match_reference_bodies(O, case):
    g = load(case)
    opt = O.scatter(g["crd"], g["tet"])
    assert np.max(np.abs(opt - g["opt"])) <= 1e-6
    deg, full = O.ball_codes(len(g["crd"]), g["tet"])
    new, res = O.gather(g["crd"], deg, full, opt)
    assert np.max(np.abs(new - g["newcrd"])) <= 1e-6
    assert np.max(np.abs(res - g["res"])) <= 1e-7


@pytest.mark.parametrize("case", CASES)
def test_fixture_tables_are_the_reference_hosts(case):
    """The integer tables stored with these fixtures equal the ones the
    reference's own host library built for the same mesh
    (refhost_<case>, made by make_refhost.py), except row 0 of the high
    table, which the reference leaves unwritten."""
    g, r = load(case), load("refhost_" + case)
    assert np.array_equal(g["deg"], r["deg"])
    assert np.array_equal(g["base"][:int(r["n_base"])], r["base"])
    assert len(g["high"]) == int(r["n_high"])
    if len(r["high"]):
        assert np.array_equal(g["high"][1:], r["high"][1:]) and not r["high"][0].any()
    assert np.array_equal(g["edges"], r["edges"])


def test_ball_known_answer(O):
    """Two tets sharing face (1,2,3): the ball lists elements in descending
    index order with codes (element << 4) | local index."""
    tet = np.array([[0, 1, 2, 3], [4, 3, 2, 1]], np.int32)
    deg, mp, hs, base, high = O.ver_tet_ball(5, tet, 32, 64)
    assert deg.tolist() == [1, 2, 2, 2, 1]
    assert mp == 5 and hs == 0
    assert base[0, :1].tolist() == [(0 << 4) | 0]
    assert base[1, :2].tolist() == [(1 << 4) | 3, (0 << 4) | 1]
    assert base[2, :2].tolist() == [(1 << 4) | 2, (0 << 4) | 2]
    assert base[3, :2].tolist() == [(1 << 4) | 1, (0 << 4) | 3]
    assert base[4, :1].tolist() == [(1 << 4) | 0]
    assert not base[0, 1:].any()


def test_edges_known_answer(O):
    """Edges in order of first appearance, local order (0,1) (1,2) (2,0)
    (3,0) (3,1) (3,2), stored (min, max)."""
    tet = np.array([[0, 1, 2, 3], [4, 3, 2, 1]], np.int32)
    e = O.tet_edges(tet).tolist()
    assert e == [[0, 1], [1, 2], [0, 2], [0, 3], [1, 3], [2, 3], [3, 4], [2, 4], [1, 4]]


def test_high_degree_split(O):
    """Reflected split: degrees up to 48 need the 64-wide high table; line
    MaxPos is the first line above 32 and its full ball is in high row 0."""
    g = load("reflected_n6.npz")
    deg, mp, hs, base, high = O.ver_tet_ball(len(g["crd"]), g["tet"], 32, 64)
    assert hs == 64
    assert deg[:mp].max() <= 32 and deg[mp] > 32
    codes = high[0, :deg[mp]]
    assert np.all(np.diff(codes >> 4) < 0)          # descending elements
    assert not high[0, deg[mp]:].any()
    assert np.array_equal(base[mp], high[0, :32])


@pytest.mark.parametrize("op", range(7))
def test_reduce_known_answers(O, op):
    x = np.array([3.0, -1.5, 0.0, 2.25, -4.0], np.float32)
    expect = [-4.0, 3.0, -0.25, 4.0, 10.75, 9 + 2.25 + 5.0625 + 16, 4.0][op]
    assert O.reduce(op, x) == pytest.approx(expect, abs=1e-12)


def test_mean_ratio_regular_tet(O):
    s = np.sqrt(2.0)
    crd = np.array([[1, 0, -1 / s, 0], [-1, 0, -1 / s, 0], [0, 1, 1 / s, 0], [0, -1, 1 / s, 0]],
                   np.float32)
    tet = np.array([[0, 1, 2, 3]], np.int32)
    q = O.mean_ratio(crd, tet)
    assert abs(abs(q[0]) - 1.0) < 1e-6
    q2 = O.mean_ratio(crd, tet[:, [0, 2, 1, 3]])
    assert q2[0] == pytest.approx(-q[0])


def test_refcl_fresh_mesh(O, G):
    """Where the reference tree is present, its bodies and the oracle agree
    on a mesh that is not in the fixtures."""
    if O.refcl() is None:
        pytest.skip("reference tree not present")
    crd, tet, ref = G.cube_mesh(7, split=1, jitter=0.3, seed=99)
    q = O.quality_ref(crd, tet)
    qr = O.ref_quality(crd, tet)
    assert np.max(np.abs(q - qr)) <= 1e-6 * np.max(np.abs(q))


# P2 quality: FP64 restatement against the reference body evaluated in FP32;
# the tolerance covers the FP32 rounding of the triple products and roots
P2_ATOL, P2_RTOL = 2e-6, 1e-4


def test_p2_quality_matches_reference_body(O):
    g = load("p2_n5.npz")
    q = O.p2_quality(g["crd"], g["mid"], g["tet"], g["tedg"])
    assert np.all(np.abs(q - g["quality"]) <= P2_ATOL + P2_RTOL * np.abs(q))
    assert (q < 0).any() and (q > 0.5).any()     # the fixture has inverted and good elements


def test_p2_quality_known_answers(O):
    """Straight P2 tets (mid-edge nodes at the midpoints): the Jacobian is
    constant and V2 = V1, so q is the shape factor 2 sqrt(6) V / (L S) with
    V = 6 vol, S = 2 area sum; 1 for the regular tetrahedron; curving an edge
    outward lowers it."""
    s = np.sqrt(2.0)
    crd = np.array([[1, 0, -1 / s, 0], [-1, 0, -1 / s, 0], [0, 1, 1 / s, 0], [0, -1, 1 / s, 0]],
                   np.float32)
    tet = np.array([[0, 1, 2, 3]], np.int32)
    if np.linalg.det(crd[1:, :3] - crd[0, :3]) < 0:
        tet = tet[:, [0, 2, 1, 3]]
    loc = [(0, 1), (1, 2), (2, 0), (3, 0), (3, 1), (3, 2)]
    mid = np.zeros((6, 4), np.float32)
    for e, (a, b) in enumerate(loc):
        mid[e, :3] = 0.5 * (crd[tet[0, a], :3] + crd[tet[0, b], :3])
    tedg = np.arange(6, dtype=np.int32)[None, :]
    q = O.p2_quality(crd, mid, tet, tedg)
    assert q[0] == pytest.approx(1.0, abs=1e-6)
    # a right-angle corner tet: shape factor by hand
    crd2 = np.array([[0, 0, 0, 0], [1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)
    mid2 = np.zeros((6, 4), np.float32)
    for e, (a, b) in enumerate(loc):
        mid2[e, :3] = 0.5 * (crd2[a, :3] + crd2[b, :3])
    q2 = O.p2_quality(crd2, mid2, np.array([[0, 1, 2, 3]], np.int32), tedg)
    area = 3 * 0.5 + np.sqrt(3) / 2
    assert q2[0] == pytest.approx(2 * np.sqrt(6) * 1.0 / (np.sqrt(2) * 2 * area), rel=1e-12)
    mid2[1, :3] += 0.05                          # edge (1,2) bent outward
    q3 = O.p2_quality(crd2, mid2, np.array([[0, 1, 2, 3]], np.int32), tedg)
    assert 0 < q3[0] < q2[0]


def test_p2_refcl_fresh_mesh(O, G):
    if O.refcl() is None:
        pytest.skip("reference tree not present")
    crd, tet, edges, mid, tedg = G.p2_mesh(6, split=0, jitter=0.25, curve=0.1, seed=5)
    q = O.p2_quality(crd, mid, tet, tedg)
    qr = O.ref_p2_quality(crd, mid, tet, tedg)
    assert np.all(np.abs(q - qr) <= P2_ATOL + P2_RTOL * np.abs(q))
