"""The no-allocation plain render (pbr_plain_render_noalloc) against the
existing plain path (pbr_plain_clear / pbr_plain_draw / pbr_plain_resolve,
whose buffer is cudaMalloc'd), called through the C ABI, twice in a row.

Callers that may not allocate device memory while rendering (during a CUDA
stream capture, or under a framework allocator that owns the device memory)
use the no-allocation entry point; its scratch is a static device array of
16 MiB, so requests beyond about 2M pixels are rejected.  After the first
call on a device (which loads the module holding that array), further calls
leave the device's free memory unchanged.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import pytest
import torch

from pybatchrender_gb300 import _capi, workloads

pytestmark = pytest.mark.gpu


def _plain_reference(r, out, depth, stream):
    _capi.call(r._lib, r._ctx, "pbr_plain_clear", stream)
    for nid in r._node_ids.values():
        _capi.call(r._lib, r._ctx, "pbr_plain_draw", nid, stream)
    _capi.call(r._lib, r._ctx, "pbr_plain_resolve", _capi.ptr(out), _capi.ptr(depth), stream)


@pytest.mark.parametrize("kernel", ["auto", "tile"])
def test_noalloc_matches_plain_path(cuda, kernel):
    r = workloads.cartpole_bench(num_scenes=96, res=64, seed=41, raster_kernel=kernel)
    stream = torch.cuda.current_stream().cuda_stream
    shape = (96, 3, 64, 64)
    for call in range(2):  # two calls in a row: the shared scratch keeps the last call's contents
        r._step(workloads.cartpole_states(96, seed=42 + call, device=cuda))
        ref_out = torch.empty(shape, dtype=torch.uint8, device=cuda)
        ref_depth = torch.empty((96, 64, 64), dtype=torch.float32, device=cuda)
        _plain_reference(r, ref_out, ref_depth, stream)
        out = torch.full(shape, 7, dtype=torch.uint8, device=cuda)
        depth = torch.full((96, 64, 64), -1.0, dtype=torch.float32, device=cuda)
        _capi.call(r._lib, r._ctx, "pbr_plain_render_noalloc", _capi.ptr(out), _capi.ptr(depth), stream)
        torch.cuda.synchronize()
        assert torch.equal(out, ref_out), f"call {call}"
        assert torch.equal(depth, ref_depth), f"call {call}"
        assert torch.equal(out, r.render())  # and the batched path


def test_noalloc_rejects_oversized_requests(cuda):
    r = workloads.cartpole_bench(num_scenes=640, res=64, seed=43)
    out = torch.empty((640, 3, 64, 64), dtype=torch.uint8, device=cuda)
    rc = r._lib.pbr_plain_render_noalloc(r._ctx, _capi.ptr(out), None, torch.cuda.current_stream().cuda_stream)
    assert rc == _capi.PBR_ERR_CAPACITY
    assert b"static buffer" in r._lib.pbr_last_error(r._ctx)


def test_noalloc_leaves_device_memory_unchanged(cuda):
    """Free device memory (cudaMemGetInfo) is the same before and after three
    calls that follow the first one: no call reserves device memory.  Every
    tensor the calls touch exists before the first reading."""
    r = workloads.cartpole_bench(num_scenes=96, res=64, seed=44)
    r._step(workloads.cartpole_states(96, seed=45, device=cuda))
    stream = torch.cuda.current_stream().cuda_stream
    out = torch.empty((96, 3, 64, 64), dtype=torch.uint8, device=cuda)
    depth = torch.empty((96, 64, 64), dtype=torch.float32, device=cuda)
    _capi.call(r._lib, r._ctx, "pbr_plain_render_noalloc", _capi.ptr(out), _capi.ptr(depth), stream)
    torch.cuda.synchronize()
    first = out.clone()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _capi.call(r._lib, r._ctx, "pbr_plain_render_noalloc", _capi.ptr(out), _capi.ptr(depth), stream)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    assert torch.equal(out, first)


def test_noalloc_inside_cuda_graph_capture(cuda):
    """The entry point's main use: captured inside a CUDA stream capture (one
    eager call first loads the module that holds the static scratch), then
    replayed after the scene state changed in place; each replay equals the
    plain path on that state."""
    r = workloads.cartpole_bench(num_scenes=96, res=64, seed=46)
    r._step(workloads.cartpole_states(96, seed=47, device=cuda))
    out = torch.empty((96, 3, 64, 64), dtype=torch.uint8, device=cuda)
    depth = torch.empty((96, 64, 64), dtype=torch.float32, device=cuda)
    _capi.call(r._lib, r._ctx, "pbr_plain_render_noalloc", _capi.ptr(out), _capi.ptr(depth),
               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        _capi.call(r._lib, r._ctx, "pbr_plain_render_noalloc", _capi.ptr(out), _capi.ptr(depth),
                   torch.cuda.current_stream().cuda_stream)
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (48, 49):
        r._step(workloads.cartpole_states(96, seed=seed, device=cuda))
        g.replay()
        ref_out = torch.empty_like(out)
        ref_depth = torch.empty_like(depth)
        _plain_reference(r, ref_out, ref_depth, stream)
        torch.cuda.synchronize()
        assert torch.equal(out, ref_out), seed
        assert torch.equal(depth, ref_depth), seed
