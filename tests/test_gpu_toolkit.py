"""Every function of the geometric toolkit on the GPU against the
reference's own sources/toolkit.cl run on the CPU.

tests/kernels/toolkit_table.cl calls each toolkit function on a jittered
hexahedron and stores 60 results.  tests/golden/toolkit.npz holds 512 such
hexahedra and the results of that body compiled against the reference's
toolkit (oracle/refcl, tests/golden/make_golden.py).  Here the same body is
compiled by GmlCompileKernel against this library's toolkit and run on the
GPU.  Tolerance: 2e-5 of max(1, |value|) (FP32, the GPU contracting products
into FMAs), 1e-3 for the line and plane intersections, whose divisions by
small dot products amplify rounding."""
import os

import numpy as np
import pytest

from conftest import PARAMS

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")

NAMES = (["DisPow", "CalLen", "CalSrf", "CalVol", "CalEdgLen", "CalTriSrf", "CalQadSrf",
          "CalTetVol", "CalPyrVol", "CalPriVol", "CalHexVol", "CalTriQal", "CalQadQal",
          "CalTetQal", "CalPyrQal", "CalPriQal", "CalHexQal", "DisVerLin", "DisVerPla",
          "DisVerEdg"]
         + ["%s.%s" % (f, c) for f in ("GetEdgTng", "GetTriNrm", "GetQadNrm", "PrjVerLin",
                                        "PrjVerPla", "LinIntLin", "LinIntPla", "PlaIntPla.crd",
                                        "PlaIntPla.tng", "MulMatVec") for c in "xyzw"])
LOOSE = {n for n in NAMES if n.startswith(("LinIntLin", "LinIntPla", "PlaIntPla"))}


def test_toolkit_functions_match_reference(G, gpu):
    gd = dict(np.load(os.path.join(GOLD, "toolkit.npz")))
    pts, ref = gd["pts"], gd["res"]
    n = len(pts)
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    v = G.lib.GmlNewMeshData(gpu, G.GmlVertices, n)
    assert v > 0
    G.set_data(gpu, v, np.zeros((n, 4), np.float32))
    p = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 8, G.GmlFlt4, b"Pts")
    r = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 64, G.GmlFlt, b"Res")
    assert p > 0 and r > 0
    G.set_data(gpu, p, pts)
    with open(os.path.join(KDIR, "toolkit_table.cl"), "rb") as f:
        src = f.read()
    k = G.compile_kernel(gpu, src, "toolkit_table", G.GmlVertices,
                         [(p, G.GmlReadMode, 0), (r, G.GmlWriteMode, 0)])
    assert k > 0 and G.lib.GmlLaunchKernel(gpu, k) == 1
    got = G.get_data(gpu, r, np.float32, (n, 64))
    bad = []
    for c, name in enumerate(NAMES):
        tol = (1e-3 if name in LOOSE else 2e-5) * np.maximum(1.0, np.abs(ref[:, c]))
        err = np.abs(got[:, c].astype(np.float64) - ref[:, c])
        if not np.all(err <= tol):
            bad.append((name, float(err.max())))
    assert not bad, bad
    assert np.all(got[:, len(NAMES):] == 0)
