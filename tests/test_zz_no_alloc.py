"""rt_morton_sort_noalloc: the Morton sort for callers that cannot allocate device memory
(a plugin whose host application owns and budgets the device memory, or a latency-bound
path where cudaMalloc / cudaFree would block). It works on device buffers the caller owns and
a fixed static device array, and must give exactly what the allocating rt_morton_sort gives.
Collected last (file name) so a stop-at-first-failure run has run every other test first."""
import numpy as np
import pytest

import raytrace_gb300 as rt

pytestmark = pytest.mark.gpu


def _noalloc(torch, tri: np.ndarray):
    n = tri.shape[0]
    d_tri = torch.from_numpy(np.ascontiguousarray(tri, np.float32)).cuda()
    d_codes = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = rt.lib.rt_morton_sort_noalloc(d_tri.data_ptr(), n, d_codes.data_ptr(), d_perm.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, d_codes.cpu().numpy().view(np.uint32), d_perm.cpu().numpy().view(np.uint32)


def test_noalloc_matches_allocating_sort_twice_in_a_row():
    torch = pytest.importorskip("torch")
    with rt.Context(0) as ctx:
        rng = np.random.default_rng(12)
        big = rng.normal(size=(200_000, 9)).astype(np.float32)
        small = rt.SceneHost.config(3, 0).tri_points()[:30_000]   # second call: fewer triangles
        small = np.concatenate([small, small[:500]])              # with duplicated codes
        for tri in (big, small):
            rc, codes, perm = _noalloc(torch, tri)
            assert rc == rt.RT_OK
            ref_codes, ref_perm = ctx.morton_sort(tri)
            np.testing.assert_array_equal(codes, ref_codes)
            np.testing.assert_array_equal(perm, ref_perm)


def test_noalloc_at_capacity_matches_and_allocates_nothing():
    """Exactly RT_NOALLOC_MAX_TRIS triangles (the fixed array's layout is tight there) against the
    allocating sort; after a first call has loaded the array, a second call changes neither the
    device's free memory nor torch's allocated bytes."""
    torch = pytest.importorskip("torch")
    n = rt.RT_NOALLOC_MAX_TRIS
    tri = np.random.default_rng(99).uniform(-50, 50, size=(n, 9)).astype(np.float32)
    d_tri = torch.from_numpy(tri).cuda()
    d_codes = torch.empty(n, dtype=torch.int32, device="cuda")
    d_perm = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        d_codes.fill_(-1)
        d_perm.fill_(-1)
        rc = rt.lib.rt_morton_sort_noalloc(d_tri.data_ptr(), n, d_codes.data_ptr(), d_perm.data_ptr(), stream)
        torch.cuda.synchronize()
        return rc

    assert call() == rt.RT_OK   # first call on the device: loads the library's array
    free0, allocated0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    assert call() == rt.RT_OK
    free1, allocated1 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    assert (free1, allocated1) == (free0, allocated0)
    with rt.Context(0) as ctx:
        ref_codes, ref_perm = ctx.morton_sort(tri)
    np.testing.assert_array_equal(d_codes.cpu().numpy().view(np.uint32), ref_codes)
    np.testing.assert_array_equal(d_perm.cpu().numpy().view(np.uint32), ref_perm)


def test_noalloc_rejects_inputs_beyond_capacity():
    torch = pytest.importorskip("torch")
    n = rt.RT_NOALLOC_MAX_TRIS + 1
    d = torch.zeros(16, dtype=torch.float32, device="cuda")   # never read: the size check comes first
    rc = rt.lib.rt_morton_sort_noalloc(d.data_ptr(), n, d.data_ptr(), d.data_ptr(), None)
    assert rc == rt.RT_ERR_TOO_LARGE
