"""Morton sort through the entry point that allocates no device memory.

apic_morton_sort_noalloc serves callers that cannot allocate device memory
(work recorded into a stream capture, or an application whose device memory
is owned by another runtime or a fixed budget): its scratch is a fixed array
inside the library, and the caller supplies the input and output buffers.
This test gives it device buffers that the test itself allocates and checks
two consecutive calls, on two different particle sets, bit for bit against
the handle-based sort (APIC_STAGE_SORT), which allocates its own scratch.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import apic_gb300 as A

pytestmark = pytest.mark.gpu


def _handle_sort(side, px, py):
    g = A.Apic(side, side, 1.0 / side, A.WorldProperties())
    g.set_particles(px, py)
    g.run_stage("sort", 0.0)
    keys, vals = g.read_field("sort_keys"), g.read_field("sort_vals")
    g.close()
    return keys, vals


def test_noalloc_sort_matches_handle_sort(gpu_lib):
    if A.device_count() == 0:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    lib = A.load_library()
    cases = [
        (256, A.scene_params(A.SCENE_DAM_BREAK_DISK, 256, cell_size=1 / 256, sub=2, seed=1, fluid_x=0.5,
                             fluid_y=0.5, disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))),
        (512, A.scene_params(A.SCENE_NOISE, 512, cell_size=1 / 512, sub=2, seed=2, noise_period=0.1,
                             noise_threshold=0.5, vel_sigma=0.5)),
    ]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for side, scene in cases:  # two calls in a row
        px, py, _, _ = A.generate_scene(scene)
        n = len(px)
        ref_keys, ref_vals = _handle_sort(side, px, py)
        dpx = torch.from_numpy(px).cuda()
        dpy = torch.from_numpy(py).cuda()
        keys = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        vals = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.apic_morton_sort_noalloc(dpx.data_ptr(), dpy.data_ptr(), n, side, side, 1.0 / side,
                                          keys.data_ptr(), vals.data_ptr(), stream)
        assert rc == A.OK, lib.apic_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(keys.cpu().numpy().view(np.uint32), ref_keys)
        assert np.array_equal(vals.cpu().numpy().view(np.uint32), ref_vals)


def test_noalloc_sort_at_the_scratch_limit_on_a_side_stream(gpu_lib):
    """Exactly 1,048,576 particles (the largest count the fixed scratch array
    holds, so its last word is used) on a non-default stream, twice in a row."""
    if A.device_count() == 0:
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    lib = A.load_library()
    side, n = 1024, 1 << 20
    rng = np.random.default_rng(7)
    side_stream = torch.cuda.Stream()
    for call in range(2):
        px = rng.uniform(0.0, 1.0, n).astype(np.float32)
        py = rng.uniform(0.0, 1.0, n).astype(np.float32)
        if call == 1:  # ties and cells at the clamp
            px[::3] = 0.5
            py[::5] = 1.5
        ref_keys, ref_vals = _handle_sort(side, px, py)
        with torch.cuda.stream(side_stream):
            dpx = torch.from_numpy(px).cuda()
            dpy = torch.from_numpy(py).cuda()
            keys = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            vals = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            rc = lib.apic_morton_sort_noalloc(dpx.data_ptr(), dpy.data_ptr(), n, side, side, 1.0 / side,
                                              keys.data_ptr(), vals.data_ptr(),
                                              ctypes.c_void_p(side_stream.cuda_stream))
            assert rc == A.OK, lib.apic_last_error()
        side_stream.synchronize()
        assert np.array_equal(keys.cpu().numpy().view(np.uint32), ref_keys)
        assert np.array_equal(vals.cpu().numpy().view(np.uint32), ref_vals)


def test_noalloc_sort_rejects_oversize(gpu_lib):
    lib = A.load_library()
    rc = lib.apic_morton_sort_noalloc(None, None, (1 << 20) + 1, 64, 64, 1 / 64, None, None, None)
    assert rc == A.ERR_INVALID_ARG
    assert b"1048576" in lib.apic_last_error()
    rc = lib.apic_morton_sort_noalloc(None, None, 16, 65537, 64, 1 / 64, None, None, None)
    assert rc == A.ERR_INVALID_ARG
    assert b"65536" in lib.apic_last_error()
