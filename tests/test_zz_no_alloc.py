"""The allocation-free cell sort, mpmgpu_sort_by_cell_noalloc.

It exists for callers that cannot call cudaMalloc -- for example a host that
reserves all device memory up front and may not allocate while runs are in
flight.  It must give exactly what mpmgpu_sort_by_cell gives (a stable argsort
of the element indices), call after call, even though every call reuses the
same fixed scratch array inside the library.  Kept in a file that pytest
collects last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 131072  # MPMGPU_NOALLOC_MAX_PARTICLES


def _sort(lib, fn, keys_np, nelems, torch):
    n = keys_np.size
    d_keys = torch.from_numpy(keys_np).cuda()
    d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = getattr(lib, fn)(C.c_void_p(d_keys.data_ptr()), n, nelems, C.c_void_p(d_perm.data_ptr()), None)
    assert st == 0, lib.mpmgpu_last_error(None)
    return d_perm.cpu().numpy()


def test_noalloc_sort_matches_allocating_sort_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    cases = [(MAX_N, 570000), (50001, 3000)]  # two calls in a row, the second smaller
    for n, nelems in cases:
        keys = rng.integers(0, nelems, size=n, dtype=np.int32)
        keys[: n // 4] = keys[n // 2]  # many particles in one cell
        want = _sort(gpu_lib, "mpmgpu_sort_by_cell", keys, nelems, torch)
        got = _sort(gpu_lib, "mpmgpu_sort_by_cell_noalloc", keys, nelems, torch)
        assert np.array_equal(got, want)
        assert np.array_equal(got, np.argsort(keys, kind="stable").astype(np.int32))


def test_noalloc_sort_rejects_too_many_particles(gpu_lib):
    torch = pytest.importorskip("torch")
    n = MAX_N + 1
    d_keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = gpu_lib.mpmgpu_sort_by_cell_noalloc(C.c_void_p(d_keys.data_ptr()), n, 10, C.c_void_p(d_perm.data_ptr()),
                                             None)
    assert st == 1
    assert b"exceeds the maximum" in gpu_lib.mpmgpu_last_error(None)
