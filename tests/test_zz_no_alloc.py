"""The allocation-free force-sum entry point (ibm_force_sums_noalloc), through the C ABI.

Callers that cannot call cudaMalloc at the time they need the lift/drag sums -- a
real-time loop with a fixed device memory budget, or a host whose device memory belongs to
a pool allocator it cannot reach -- pass their own device arrays and get the sums back
without the library allocating anything; its scratch is a fixed device array built into
the library. The call is synchronous, so it refuses a stream that is being captured into a
CUDA graph. This file is collected last, so a failure here comes after every other test
has run.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_force_sums_without_allocation_match_ibm_history(built_pkg):
    torch = pytest.importorskip("torch")
    pkg = built_pkg
    lib = pkg.lib()
    cfg = pkg.wing_case(64, 32, 6, 10.0, re=30.0)
    sim = pkg.Simulation(cfg)
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for step in (1, 2):   # two calls in a row, each on the forces of a new step
        sim.step_host_motion(step)
        want = sim.ibm.force_history(1)[0]          # the existing entry point's sums
        fx, fy, _ = sim.ibm.read_forces()
        mk = sim.ibm.read_markers()
        d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda()
             for k, v in (("fx", fx), ("fy", fy), ("FXk", mk["FXk"]), ("FYk", mk["FYk"]))}
        torch.cuda.synchronize()
        out = np.zeros(4, np.float64)
        rc = lib.ibm_force_sums_noalloc(_dptr(d["fx"]), _dptr(d["fy"]), nx, ny, nz,
                                        _dptr(d["FXk"]), _dptr(d["FYk"]), cfg.n_markers, stream,
                                        out.ctypes.data_as(ctypes.c_void_p))
        assert rc == 0, lib.clbm_last_error()
        assert np.any(out != 0.0)
        np.testing.assert_allclose(out, want, rtol=1e-10, atol=1e-12)
    sim.close()


def test_force_sums_without_allocation_reject_oversize(built_pkg):
    torch = pytest.importorskip("torch")
    lib = built_pkg.lib()
    buf = torch.zeros(16, device="cuda")
    out = np.zeros(4, np.float64)
    rc = lib.ibm_force_sums_noalloc(_dptr(buf), _dptr(buf), 4096, 4096, 5, None, None, 0, None,
                                    out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 2
    assert b"exceed the maximum" in lib.clbm_last_error()


MAX_CELLS = 16384 * 4096   # the fixed scratch covers this many cells


def test_force_sums_without_allocation_accept_exactly_the_maximum(built_pkg):
    torch = pytest.importorskip("torch")
    lib = built_pkg.lib()
    buf = torch.zeros(MAX_CELLS, device="cuda")   # 256 MB of zero forces
    buf[7] = 0.01
    buf[MAX_CELLS - 1] = 0.5                      # clipped to 0.05 by the sums
    torch.cuda.synchronize()
    out = np.zeros(4, np.float64)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ibm_force_sums_noalloc(_dptr(buf), _dptr(buf), 4096, 4096, 4, None, None, 0, stream,
                                    out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0, lib.clbm_last_error()
    want = float(np.float32(0.01)) + float(np.float32(0.05))
    np.testing.assert_allclose(out, [want, want, 0.0, 0.0], rtol=1e-12, atol=0)
    rc = lib.ibm_force_sums_noalloc(_dptr(buf), _dptr(buf), MAX_CELLS + 1, 1, 1, None, None, 0,
                                    stream, out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 2
    assert b"exceed the maximum" in lib.clbm_last_error()


def test_force_sums_without_allocation_refuse_a_capturing_stream(built_pkg):
    torch = pytest.importorskip("torch")
    lib = built_pkg.lib()
    buf = torch.full((64,), 0.01, device="cuda")
    x = torch.ones(8, device="cuda")
    torch.cuda.synchronize()
    out = np.zeros(4, np.float64)
    outp = out.ctypes.data_as(ctypes.c_void_p)
    # outside capture the call works (and makes the one-time set-up on this device)
    rc = lib.ibm_force_sums_noalloc(_dptr(buf), _dptr(buf), 4, 4, 4, None, None, 0,
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), outp)
    assert rc == 0, lib.clbm_last_error()
    np.testing.assert_allclose(out[:2], 64 * float(np.float32(0.01)), rtol=1e-12)
    out[:] = -1.0
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        cap = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        rc = lib.ibm_force_sums_noalloc(_dptr(buf), _dptr(buf), 4, 4, 4, None, None, 0, cap, outp)
        msg = lib.clbm_last_error()
        y = x * 3.0
    assert rc == 4, msg
    assert b"captured" in msg
    assert np.all(out == -1.0)          # nothing was written
    g.replay()                          # the caller's capture is still valid
    torch.cuda.synchronize()
    assert torch.equal(y, torch.full_like(x, 3.0))
    # and the entry point still works afterwards
    rc = lib.ibm_force_sums_noalloc(_dptr(buf), _dptr(buf), 4, 4, 4, None, None, 0,
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), outp)
    assert rc == 0, lib.clbm_last_error()
    np.testing.assert_allclose(out[:2], 64 * float(np.float32(0.01)), rtol=1e-12)
