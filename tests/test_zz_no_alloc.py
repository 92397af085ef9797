"""cf_cull_lights_static_scratch: culling for callers that cannot allocate.

A caller that records its frame where device allocation is off limits (inside
a host allocator's critical section, in a plugin whose device memory its host
reserves up front, or in a real-time loop that cannot pay for cudaMalloc and
the synchronisation of cudaFree) cannot hand cf_cull_lights a workspace.  The
static-scratch entry point takes the same inputs and outputs and uses a fixed
32 MiB device array of the library instead.  These tests call it through the C
ABI twice in a row, on views of different sizes, and require the same cells,
index list and total as cf_cull_lights with a workspace and as the oracle —
bit for bit, the tolerance of every culling test here — with and without a
caller error word.  This file is collected last so that a run stopping at its
first failure has run everything else first.
"""
import ctypes as C

import numpy as np
import pytest

from hellovulkan_gb300 import scenes

pytestmark = pytest.mark.gpu


def _inputs(view):
    import torch
    from hellovulkan_gb300._lib import check, lib
    n = view.clusters
    aabbs = torch.empty(n * 8, dtype=torch.float32, device="cuda")
    check(lib().cf_generate_aabbs(C.byref(view.ubo), aabbs.data_ptr(), torch.cuda.current_stream().cuda_stream))
    lights = torch.from_numpy(np.ascontiguousarray(view.lights)).cuda()
    return aabbs, lights


def _outputs(view):
    import torch
    n, cap = view.clusters, view.cap
    return (torch.full((n * 2,), -1, dtype=torch.int32, device="cuda"),
            torch.full((n * cap,), -1, dtype=torch.int32, device="cuda"),
            torch.full((1,), -1, dtype=torch.int32, device="cuda"))


def _read(view, cells, idx, total):
    import torch
    torch.cuda.synchronize()
    t = int(total.item())
    return cells.cpu().numpy().view(np.uint32).reshape(view.clusters, 2), idx[:t].cpu().numpy().view(np.uint32), t


def _with_workspace(view, aabbs, lights):
    import torch
    from hellovulkan_gb300._lib import check, lib
    cells, idx, total = _outputs(view)
    nbytes = C.c_uint64()
    check(lib().cf_cull_workspace_size(C.byref(view.ubo), view.light_count, view.cap, C.byref(nbytes)))
    ws = torch.zeros(nbytes.value, dtype=torch.uint8, device="cuda")
    check(lib().cf_cull_lights(C.byref(view.ubo), aabbs.data_ptr(), lights.data_ptr(), view.light_count, view.cap,
                               cells.data_ptr(), idx.data_ptr(), view.clusters * view.cap, total.data_ptr(),
                               ws.data_ptr(), nbytes.value, torch.cuda.current_stream().cuda_stream))
    return _read(view, cells, idx, total)


def _with_static_scratch(view, aabbs, lights, error_word=True):
    import torch
    from hellovulkan_gb300._lib import check, lib
    cells, idx, total = _outputs(view)
    err = torch.zeros(1, dtype=torch.int32, device="cuda") if error_word else None
    check(lib().cf_cull_lights_static_scratch(C.byref(view.ubo), aabbs.data_ptr(), lights.data_ptr(),
                                              view.light_count, view.cap, cells.data_ptr(), idx.data_ptr(),
                                              view.clusters * view.cap, total.data_ptr(),
                                              err.data_ptr() if error_word else None,
                                              torch.cuda.current_stream().cuda_stream))
    out = _read(view, cells, idx, total)
    if error_word:
        assert int(err.item()) == 0
    return out


def _oracle(oracle, view, aabbs):
    a = aabbs.cpu().numpy().reshape(view.clusters, 8)
    assert np.array_equal(a.view(np.uint32), oracle.generate_aabbs(view.ubo).view(np.uint32))
    cells, idx, _ = oracle.cull(view.ubo, a, view.lights, view.cap)
    return cells, idx


def test_static_scratch_matches_the_workspace_entry_point_on_two_calls_in_a_row(cflib, oracle):
    import torch
    assert torch.cuda.is_available()
    # the larger view first, so the second call runs over the first one's leftovers
    for view in (scenes.plain_large(2), scenes.plain_small(1)):
        aabbs, lights = _inputs(view)
        want_cells, want_idx, want_total = _with_workspace(view, aabbs, lights)
        got_cells, got_idx, got_total = _with_static_scratch(view, aabbs, lights)
        assert got_total == want_total
        assert np.array_equal(got_cells, want_cells)
        assert np.array_equal(got_idx, want_idx)
        o_cells, o_idx = _oracle(oracle, view, aabbs)
        assert np.array_equal(got_cells, o_cells) and np.array_equal(got_idx, o_idx)


def test_static_scratch_without_a_caller_error_word(cflib, oracle):
    """No d_device_error: the call clears the array's own word and the
    kernels report into it; the results are the same as with a word."""
    for view in (scenes.plain_small(3), scenes.plain_large(4, n_lights=4000)):
        aabbs, lights = _inputs(view)
        for _ in range(2):
            got_cells, got_idx, got_total = _with_static_scratch(view, aabbs, lights, error_word=False)
            o_cells, o_idx = _oracle(oracle, view, aabbs)
            assert got_total == o_idx.size
            assert np.array_equal(got_cells, o_cells) and np.array_equal(got_idx, o_idx)


def test_static_scratch_rejects_views_that_do_not_fit(cflib):
    from hellovulkan_gb300._lib import lib
    view = scenes.custom_view((64, 64, 64), 4096, 4096, 0.1, 100.0)
    st = lib().cf_cull_lights_static_scratch(C.byref(view.ubo), C.c_void_p(256), None, 0, 150, C.c_void_p(256),
                                             C.c_void_p(256), 64 ** 3 * 150, None, None, None)
    assert st == 4  # CF_ERROR_CAPACITY, before any GPU work
    assert b"static scratch" in lib().cf_last_error_message()
