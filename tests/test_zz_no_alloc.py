"""csp_trace_noalloc, the entry point that allocates nothing, for callers that cannot call cudaMalloc
(a framework whose allocator already owns the device memory; a real-time tracking loop that cannot
take cudaMalloc's synchronisation).  Checked through the C ABI against csp_trace_into on a handle with
the same scene: the records must be bit-identical, on calls made back to back with different scenes
(the fixed scratch array is shared by every call).  This file is collected last on purpose."""
import numpy as np
import pytest

from optixsoltracedemos_gb300 import native, scenes

pytestmark = pytest.mark.gpu


def _records_via_handle(torch, sc, n, seed, instance):
    t = native.tracer_for(sc, seed=seed, instance=instance, num_rays=n)
    hits = torch.empty(n * 5 * 4, dtype=torch.float32, device="cuda")
    ids = torch.empty(n * 5, dtype=torch.int32, device="cuda")
    t.trace_into(hits.data_ptr(), ids.data_ptr(), 0, n, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    t.close()
    return hits.cpu().numpy().view(np.uint32), ids.cpu().numpy().view(np.uint32)


def _records_noalloc(torch, sc, n, seed, instance, first=0):
    # outputs are owned by the caller; fill them with garbage so a partial write would show
    hits = torch.full((n * 5 * 4,), float("nan"), dtype=torch.float32, device="cuda")
    ids = torch.full((n * 5,), 12345, dtype=torch.int32, device="cuda")
    native.trace_noalloc(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, hits.data_ptr(), ids.data_ptr(),
                         first_ray=first, num_rays=n, seed=seed, instance=instance, device=0,
                         stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return hits.cpu().numpy().view(np.uint32), ids.cpu().numpy().view(np.uint32)


def test_noalloc_matches_handle_on_consecutive_calls(gpu):
    torch = pytest.importorskip("torch")
    n = 1 << 17
    runs = [(scenes.three_heliostats(), 3, 1),
            (scenes.single_parabolic(), 9, 0),
            (scenes.corridor(slope_error=1e-3), 5, 2),
            (scenes.three_heliostats(), 3, 1)]
    for sc, seed, inst in runs:
        h_ref, i_ref = _records_via_handle(torch, sc, n, seed, inst)
        h, i = _records_noalloc(torch, sc, n, seed, inst)
        np.testing.assert_array_equal(h, h_ref)   # bit-identical records
        np.testing.assert_array_equal(i, i_ref)
        assert (h_ref.view(np.float32).reshape(n, 5, 4)[:, :, 0] > 0).any()


def test_noalloc_ray_window_and_limits(gpu):
    torch = pytest.importorskip("torch")
    sc = scenes.single_parabolic()
    n_all = 1 << 16
    h_all, _ = _records_via_handle(torch, sc, n_all, 0, 0)
    h_win, _ = _records_noalloc(torch, sc, 4096, 0, 0, first=50000)
    np.testing.assert_array_equal(h_win, h_all[50000 * 20:(50000 + 4096) * 20])
    big = scenes.large_field(n_heliostats=8)  # 9 elements: over the fixed array's limit
    out = torch.empty(16 * 5 * 4, dtype=torch.float32, device="cuda")
    with pytest.raises(native.CspError) as e:
        native.trace_noalloc(big.elements, big.sun_dir, big.sun_shape, big.sun_param, out.data_ptr(), num_rays=16)
    assert e.value.status == -1 and "8 elements" in str(e.value)


def test_noalloc_allocates_no_device_memory(gpu):
    """The property the entry point exists for: after a first call (which loads the kernels and
    looks up the scratch array's address), further calls leave the device's free memory unchanged --
    no cudaMalloc, no Halton table, no staging buffer."""
    torch = pytest.importorskip("torch")
    sc = scenes.single_parabolic()
    n = 1 << 16
    hits = torch.empty(n * 5 * 4, dtype=torch.float32, device="cuda")
    ids = torch.empty(n * 5, dtype=torch.int32, device="cuda")

    def call(seed):
        native.trace_noalloc(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, hits.data_ptr(), ids.data_ptr(),
                             num_rays=n, seed=seed, device=0, stream=torch.cuda.current_stream().cuda_stream)

    call(0)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for seed in (1, 2, 3):
        call(seed)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
