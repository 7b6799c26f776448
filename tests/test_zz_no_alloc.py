"""The allocation-free sum of squares (ofd_sumsq_field_noalloc) through the
C ABI, against the handle-based reduction ofd_field_sumsq on the same field
and against an FP64 sum computed on the host from the downloaded field.

Callers that cannot allocate device memory (graph capture, foreign memory
pools, allocator-free serving loops) use the no-alloc entry point; it must
give the same FP64 sums, call after call, although its scratch is a fixed
array shared by all calls, and also when the call is recorded into a CUDA
graph on the caller's stream and replayed.  This file is collected last on
purpose.

Tolerance: 1e-12 relative (FP64 sums of the same values in different orders).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _lib():
    from opesci import runtime
    lib = runtime.load_library()
    lib.ofd_sumsq_field_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p]
    lib.ofd_sumsq_field_noalloc.restype = ctypes.c_int
    lib.ofd_noalloc_last_error.restype = ctypes.c_char_p
    return lib


def _problem():
    from opesci import runtime
    from opesci.models import layered_problem
    g, media, src, wav = layered_problem(40, space_order=4, ntsteps=30, seed=21)
    sim = runtime.Simulation(runtime.config_from_grid(g))
    sim.set_coefficients_from_grid(g)
    sim.set_media(*media)
    sim.set_source(src, wav)
    sim.step(30)
    sim.sync()
    return g, sim


def _host_sumsq(a, m):
    inner = a[m:-m, m:-m, m:-m].astype(np.float64)
    return float(np.sum(inner * inner))


def test_noalloc_sumsq_matches_handle_reduction_twice():
    torch = pytest.importorskip('torch')
    lib = _lib()
    g, sim = _problem()
    level = sim.steps % 2
    ref = sim.sumsq(level)
    dims = (ctypes.c_int * 3)(*sim.dims)
    margin = g.margin.value
    dev = torch.empty(sim.dims, dtype=torch.float32, device='cuda')
    out = torch.zeros(1, dtype=torch.float64, device='cuda')
    for f in range(9):
        rc = sim.lib.ofd_download_field_device(sim.h, f, level, ctypes.c_void_p(dev.data_ptr()))
        assert rc == 0
        sim.sync()
        host = _host_sumsq(dev.cpu().numpy(), margin)
        assert abs(host - ref[f]) <= TOL * max(abs(ref[f]), 1e-300), (f, host, ref[f])
        for call in range(2):
            out.fill_(-1.0)
            torch.cuda.synchronize()
            rc = lib.ofd_sumsq_field_noalloc(ctypes.c_void_p(dev.data_ptr()), dims, margin,
                                             ctypes.c_void_p(out.data_ptr()), None)
            assert rc == 0, lib.ofd_noalloc_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            assert abs(got - ref[f]) <= TOL * max(abs(ref[f]), 1e-300), (f, call, got, ref[f])
            assert abs(got - host) <= TOL * max(abs(host), 1e-300), (f, call, got, host)
    assert ref[3] > 0
    sim.close()


def test_noalloc_sumsq_inside_graph_capture():
    """One warm-up call on the caller's stream, then the call recorded into a
    CUDA graph on that stream (where no allocation may happen) and the graph
    replayed twice."""
    torch = pytest.importorskip('torch')
    lib = _lib()
    g, sim = _problem()
    level = sim.steps % 2
    ref = sim.sumsq(level)
    dims = (ctypes.c_int * 3)(*sim.dims)
    margin = g.margin.value
    dev = torch.empty(sim.dims, dtype=torch.float32, device='cuda')
    rc = sim.lib.ofd_download_field_device(sim.h, 3, level, ctypes.c_void_p(dev.data_ptr()))
    assert rc == 0
    sim.sync()
    host = _host_sumsq(dev.cpu().numpy(), margin)
    out = torch.zeros(1, dtype=torch.float64, device='cuda')
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        rc = lib.ofd_sumsq_field_noalloc(ctypes.c_void_p(dev.data_ptr()), dims, margin,
                                         ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s.cuda_stream))
        assert rc == 0, lib.ofd_noalloc_last_error()
    s.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        rc = lib.ofd_sumsq_field_noalloc(ctypes.c_void_p(dev.data_ptr()), dims, margin,
                                         ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s.cuda_stream))
    assert rc == 0, lib.ofd_noalloc_last_error()
    for _ in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - ref[3]) <= TOL * max(abs(ref[3]), 1e-300), (got, ref[3])
        assert abs(got - host) <= TOL * max(abs(host), 1e-300), (got, host)
    del graph
    sim.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = _lib()
    dims = (ctypes.c_int * 3)(4200, 16, 16)
    out = ctypes.c_double()
    rc = lib.ofd_sumsq_field_noalloc(ctypes.c_void_p(16), dims, 2, ctypes.c_void_p(ctypes.addressof(out)), None)
    assert rc != 0
    assert b'4096' in lib.ofd_noalloc_last_error()
    dims = (ctypes.c_int * 3)(8, 50000, 50000)
    rc = lib.ofd_sumsq_field_noalloc(ctypes.c_void_p(16), dims, 2, ctypes.c_void_p(ctypes.addressof(out)), None)
    assert rc != 0
    assert b'2^31' in lib.ofd_noalloc_last_error()
