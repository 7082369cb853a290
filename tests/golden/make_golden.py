"""Generate tests/golden/*.npz from the reference's own kernel bodies.

Runs where the reference tree is present: oracle/_ref/librefcl.so compiles
sources/toolkit.cl and the MeshQuality / NodeSmoothing example bodies of the
reference as C++ and executes them on the CPU (one loop iteration per
work-item).  The fixtures store the inputs (a small jittered cube, Kuhn and
reflected splits) and the reference outputs (quality, optimal points, relaxed
coordinates, residuals) plus the ball tables built by the reference's chained
hash algorithm (oracle.c).  Tests then pin the oracle and the GPU path to
these values on machines without the reference tree.

toolkit.npz holds 512 jittered hexahedra (8 corners each, GMlib corner order)
and the 64 results per hexahedron of tests/kernels/toolkit_table.cl, every
function of the reference's sources/toolkit.cl, compiled from the reference
tree and run on the CPU.

p2_n5.npz holds a quadratic-tet mesh (gmlib_gb300.p2_mesh: vertices, unique
edges with curved mid-edge nodes, the tet -> edge table) and the quality of
the reference's examples/P2Quality/quality.cl body on it.

Usage:  python tests/golden/make_golden.py [p2|toolkit]   (one fixture only)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import gmlib_gb300 as G  # noqa: E402  (mesh generator only)
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def make(name, n, split, jitter, seed):
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=jitter, seed=seed)
    deg, mp, hs, base, high = O.ver_tet_ball(len(crd), tet, 32, 64)
    _, full = O.ball_codes(len(crd), tet)
    q = O.ref_quality(crd, tet)
    opt = O.ref_scatter(crd, tet)
    newcrd, res = O.ref_gather(crd, deg, full, opt)
    edges = O.tet_edges(tet)
    np.savez_compressed(os.path.join(OUT, name), crd=crd, tet=tet, ref=ref, deg=deg,
                        maxpos=mp, hghsiz=hs, base=base, high=high, quality=q, opt=opt,
                        newcrd=newcrd, res=res, edges=edges)
    print(name, len(crd), len(tet), "maxdeg", deg.max(), "maxpos", mp, "high", hs)


def make_p2(name, n, split, jitter, curve, seed):
    crd, tet, edges, mid, tedg = G.p2_mesh(n, split=split, jitter=jitter, curve=curve, seed=seed)
    q = O.ref_p2_quality(crd, mid, tet, tedg)
    np.savez_compressed(os.path.join(OUT, name), crd=crd, tet=tet, edges=edges, mid=mid,
                        tedg=tedg, quality=q)
    print(name, len(crd), len(tet), len(edges), "quality min %.6g mean %.6g" % (q.min(), q.mean()))


def toolkit_points(n, seed):
    """n unit hexahedra (corners 0-3 at z = 0 and 4-7 at z = 1, each face
    counter-clockwise seen from outside the bottom) jittered by +-0.2."""
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                     [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.float64)
    rng = np.random.default_rng(seed)
    pts = np.zeros((n, 8, 4), np.float32)
    pts[:, :, :3] = base[None] + rng.uniform(-0.2, 0.2, (n, 8, 3)) + rng.uniform(-5, 5, (n, 1, 3))
    return pts


def make_toolkit(name, n, seed):
    pts = toolkit_points(n, seed)
    res = O.ref_toolkit_table(pts)
    np.savez_compressed(os.path.join(OUT, name), pts=pts, res=res)
    print(name, pts.shape, res.shape)


if __name__ == "__main__":
    if O.refcl() is None:
        sys.exit("the reference tree is needed to generate the golden fixtures")
    only = sys.argv[1] if len(sys.argv) > 1 else None
    if only is None:
        make("kuhn_n5.npz", 5, 0, 0.25, 12345)
        make("reflected_n6.npz", 6, 1, 0.3, 777)
    if only in (None, "p2"):
        make_p2("p2_n5.npz", 5, 1, 0.15, 0.08, 4242)
    if only in (None, "toolkit"):
        make_toolkit("toolkit.npz", 512, 31)
