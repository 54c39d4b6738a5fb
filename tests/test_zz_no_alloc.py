"""vsrBuildTriangleBVHNoAlloc: the BVH build for callers that cannot let the
library allocate GPU memory (a host that owns a fixed GPU memory budget and
only hands in its own buffers, or a per-frame loop that must not allocate or
free mid-frame). Its temporaries live in a fixed 8 MiB buffer in the
library's device data, so this test checks that

  * two calls in a row on different triangle sets each give exactly the
    output of the allocating entry point vsrBuildTriangleBVH (the buffer is
    reused and must be re-cleared between calls),
  * the calls allocate nothing: after a first call, device free memory
    (cudaMemGetInfo) and the default stream-ordered pool's used and
    reserved bytes are the same before and after further calls, and
  * sizes above VSR_BVH_NOALLOC_MAX_TRIANGLES are refused.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes
import importlib
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAX_TRIANGLES = 65536
LIMIT_EXCEEDED = 8


def _pkg():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    return importlib.import_module("anari-visionaray_gb300")


def _lib():
    return _pkg().vsr.load_library()


def _triangles(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, (n, 1, 3))
    T = (c + rng.normal(scale=0.3, size=(n, 3, 3))).astype(np.float32)
    v1 = np.ascontiguousarray(T[:, 0])
    return v1, np.ascontiguousarray(T[:, 1] - v1), np.ascontiguousarray(T[:, 2] - v1)


def _buffers(tris_host):
    import torch
    n = len(tris_host[0])
    dv = [torch.from_numpy(a.reshape(-1)).cuda() for a in tris_host]
    nodes = torch.zeros(4 * max(n - 1, 1) * 4, dtype=torch.float32, device="cuda")
    tris = torch.zeros(3 * n * 4, dtype=torch.float32, device="cuda")
    return n, dv, nodes, tris


def _call(lib, fn, bufs):
    import torch
    n, dv, nodes, tris = bufs
    return getattr(lib, fn)(dv[0].data_ptr(), dv[1].data_ptr(), dv[2].data_ptr(), n,
                            nodes.data_ptr(), tris.data_ptr(),
                            torch.cuda.current_stream().cuda_stream)


def _build(lib, fn, tris_host):
    import torch
    bufs = _buffers(tris_host)
    rc = _call(lib, fn, bufs)
    torch.cuda.synchronize()
    return rc, bufs[2].cpu().numpy(), bufs[3].cpu().numpy()


def test_no_alloc_build_matches_allocating_build_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = _lib()
    for n, seed in ((5000, 11), (MAX_TRIANGLES, 12)):
        host = _triangles(n, seed)
        rc_ref, nodes_ref, tris_ref = _build(lib, "vsrBuildTriangleBVH", host)
        rc, nodes, tris = _build(lib, "vsrBuildTriangleBVHNoAlloc", host)
        assert rc_ref == 0 and rc == 0
        # same kernels, same inputs: the outputs are identical bit for bit
        assert np.array_equal(nodes.view(np.uint32), nodes_ref.view(np.uint32)), n
        assert np.array_equal(tris.view(np.uint32), tris_ref.view(np.uint32)), n


def test_no_alloc_build_allocates_nothing():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = _lib()
    probe = ctypes.CDLL(os.path.join(os.path.dirname(_pkg().__file__), "libvsr_probe.so"))
    probe.vsrProbeMemPoolUsage.argtypes = [ctypes.POINTER(ctypes.c_uint64)] * 2

    def usage():
        torch.cuda.synchronize()
        used, reserved = ctypes.c_uint64(), ctypes.c_uint64()
        assert probe.vsrProbeMemPoolUsage(ctypes.byref(used), ctypes.byref(reserved)) == 0
        return torch.cuda.mem_get_info()[0], used.value, reserved.value

    bufs = [_buffers(_triangles(n, seed)) for n, seed in ((MAX_TRIANGLES, 21), (20000, 22))]
    # first calls: the address set-up, and the kernels' code loaded on first launch
    for b in bufs:
        assert _call(lib, "vsrBuildTriangleBVHNoAlloc", b) == 0
    before = usage()
    for b in bufs + bufs:
        assert _call(lib, "vsrBuildTriangleBVHNoAlloc", b) == 0
    after = usage()
    assert after == before, (before, after)


def test_no_alloc_build_rejects_too_many_triangles():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = _lib()
    n = MAX_TRIANGLES + 1
    rc = lib.vsrBuildTriangleBVHNoAlloc(1, 1, 1, n, 1, 1, None)
    assert rc == LIMIT_EXCEEDED
