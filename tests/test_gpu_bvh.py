"""The device BVH build entry point (vsrBuildTriangleBVH): structure checks.

The BVH shape is free (closest hits are ordered by (t, instance, triangle)),
so the checks are structural: every triangle appears in exactly one leaf,
the leaf-ordered copy holds the input triangles bit for bit, and every
child box stored in a node contains all triangles below it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def triangles(n, seed=0):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, (n, 1, 3))
    T = (c + rng.normal(scale=0.3, size=(n, 3, 3))).astype(np.float32)
    v1 = T[:, 0]
    return np.ascontiguousarray(v1), np.ascontiguousarray(T[:, 1] - v1), np.ascontiguousarray(T[:, 2] - v1)


def build_bvh(pkg, v1, e1, e2, fn="vsrBuildTriangleBVH"):
    import torch
    lib = pkg.vsr.load_library()
    n = len(v1)
    dv = [torch.from_numpy(a.reshape(-1)).cuda() for a in (v1, e1, e2)]
    nodes = torch.zeros(4 * max(n - 1, 1) * 4, dtype=torch.float32, device="cuda")
    tris = torch.zeros(3 * n * 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = getattr(lib, fn)(dv[0].data_ptr(), dv[1].data_ptr(), dv[2].data_ptr(), n,
                          nodes.data_ptr(), tris.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, nodes.cpu().numpy().reshape(-1, 4, 4), tris.cpu().numpy().reshape(-1, 3, 4)


def check_structure(v1, e1, e2, nodes, tris):
    n = len(v1)
    local = tris[:, 0, 3].view(np.int32)
    assert sorted(local.tolist()) == list(range(n))
    assert np.array_equal(tris[:, 0, :3], v1[local])
    assert np.array_equal(tris[:, 1, :3], e1[local])
    assert np.array_equal(tris[:, 2, :3], e2[local])
    P = np.stack([tris[:, 0, :3], tris[:, 0, :3] + tris[:, 1, :3], tris[:, 0, :3] + tris[:, 2, :3]], 1)
    tlo, thi = P.min(1), P.max(1)
    seen = np.zeros(n, int)

    def visit(node):
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        nd = nodes[node]
        ch = nd[3, :2].view(np.int32)
        boxes = [((nd[0, 0], nd[0, 2], nd[2, 0]), (nd[0, 1], nd[0, 3], nd[2, 1])),
                 ((nd[1, 0], nd[1, 2], nd[2, 2]), (nd[1, 1], nd[1, 3], nd[2, 3]))]
        for c, (blo, bhi) in zip(ch, boxes):
            if c < 0:
                code = ~int(c) & 0xFFFFFFFF
                first, count = code & ((1 << 27) - 1), (code >> 27) + 1
                clo = tlo[first:first + count].min(0)
                chi = thi[first:first + count].max(0)
                seen[first:first + count] += 1
            else:
                clo, chi = visit(int(c))
            assert np.all(np.asarray(blo) <= clo) and np.all(np.asarray(bhi) >= chi)
            lo, hi = np.minimum(lo, clo), np.maximum(hi, chi)
        return lo, hi

    import sys
    sys.setrecursionlimit(10000)
    visit(0)
    assert np.all(seen == 1)


@pytest.mark.parametrize("n", [2, 3, 17, 1000, 5000])
def test_build_triangle_bvh_structure(pkg, device, n):
    v1, e1, e2 = triangles(n, seed=n)
    rc, nodes, tris = build_bvh(pkg, v1, e1, e2)
    assert rc == 0
    check_structure(v1, e1, e2, nodes, tris)


def test_build_triangle_bvh_duplicate_centroids(pkg, device):
    """Identical Morton codes (coincident triangles) still give a valid tree."""
    v1, e1, e2 = triangles(1, seed=1)
    v1, e1, e2 = (np.repeat(a, 300, axis=0) for a in (v1, e1, e2))
    rc, nodes, tris = build_bvh(pkg, v1, e1, e2)
    assert rc == 0
    check_structure(v1, e1, e2, nodes, tris)


def test_build_triangle_bvh_rejects_bad_arguments(pkg, device):
    lib = pkg.vsr.load_library()
    assert lib.vsrBuildTriangleBVH(None, None, None, 10, None, None, None) == 1
