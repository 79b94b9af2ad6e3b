"""The allocation-free voxel build (fpt_cuda_voxel_build_static).

Callers that cannot allocate device memory -- engines that own all GPU
memory through their own pool, or frame loops that cannot take the
implicit synchronisation of cudaMalloc -- pass their own device buffers.
Two calls in a row (different scenes, so stale contents of the shared
scratch array would show) must each equal the allocating entry point
fpt_cuda_voxel_build bit for bit.  This file is collected last on purpose.
"""
import numpy as np
import pytest

from fractalpathtracer_gb300 import native_ext, scenes
from tests.test_voxel_cpu import sphere_program

pytestmark = pytest.mark.gpu


def _static_build(torch, cfg, ext):
    bg = (cfg.voxel_resolution + 7) // 8
    cap = bg ** 3 * 512
    table = torch.full((bg ** 3,), -1, dtype=torch.int32, device="cuda")
    occ = torch.full((cap,), 255, dtype=torch.uint8, device="cuda")
    dist = torch.full((cap,), -1, dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    info = native_ext.voxel_build_static(cfg, ext, table.data_ptr(), table.numel(), occ.data_ptr(), dist.data_ptr(), cap)
    n = info["active_bricks"] * 512
    return (info, table.cpu().numpy().view(np.uint32), occ[:n].cpu().numpy(), dist[:n].cpu().numpy().view(np.uint16))


def test_static_build_equals_allocating_build_twice(native):
    torch = pytest.importorskip("torch")
    cases = [scenes.voxel_mandelbox(128, 8, 8), (sphere_program(64), None)]
    for cfg, ext in cases:
        ref_info = native_ext.voxel_build(cfg, ext, 8)
        rt, ro, rd, _ = native_ext.voxel_read(ref_info)
        info, t, o, d = _static_build(torch, cfg, ext)
        assert info["active_bricks"] == ref_info["active_bricks"]
        assert info["active_cells"] == ref_info["active_cells"]
        assert np.array_equal(t, rt)
        assert np.array_equal(o, ro)
        assert np.array_equal(d, rd)


def test_static_build_rejects_oversize(native):
    torch = pytest.importorskip("torch")
    cfg, ext = scenes.voxel_mandelbox(1024, 8, 8)
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(native.NativeError, match="out of range"):
        native_ext.voxel_build_static(cfg, ext, buf.data_ptr(), 16, buf.data_ptr(), buf.data_ptr(), 16)


def test_static_build_refuses_stream_capture(native):
    """The build synchronises its stream (count readback), which a graph capture cannot hold: on a capturing
    stream the call returns an error before it enqueues anything, and the caller's capture stays usable."""
    torch = pytest.importorskip("torch")
    cfg, ext = scenes.voxel_mandelbox(64, 8, 8)
    bg = (cfg.voxel_resolution + 7) // 8
    cap = bg ** 3 * 512
    table = torch.zeros(bg ** 3, dtype=torch.int32, device="cuda")
    occ = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    dist = torch.zeros(cap, dtype=torch.int16, device="cuda")
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
        with pytest.raises(native.NativeError, match="stream capture"):
            native_ext.voxel_build_static(cfg, ext, table.data_ptr(), table.numel(), occ.data_ptr(), dist.data_ptr(), cap,
                                          stream=side.cuda_stream)
        table.add_(1)   # the capture still records the caller's own work
    graph.replay()
    torch.cuda.synchronize()
    assert int(table.sum().item()) == table.numel()
