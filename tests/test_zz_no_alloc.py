"""gb300_conservation_noalloc (static device scratch, no allocation) against
gb300_conservation (caller's reduce_array), through the C ABI.

The two reductions add the same values in different orders, so their totals
agree to within 1e-12 relative (sums of at most a few million positive
terms); two calls in a row of the no-alloc form agree bit for bit.  This file
is named to run after every other GPU test and must also pass on its own.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12
GB300_ERR_ARG = 2
MAX_ROWS = 16384


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    return flow_gb300


def totals_pair(fg, nx, ny, pad, rho, e, reduce_array):
    L = fg.lib()
    out = (ctypes.c_double * 2)()
    assert L.gb300_conservation(nx, ny, pad, fg.dptr(rho), fg.dptr(e), fg.dptr(reduce_array),
                                ctypes.cast(out, ctypes.POINTER(ctypes.c_double)), 1) == 0
    ref = (out[0], out[1])
    got = []
    for _ in range(2):
        o = (ctypes.c_double * 2)(-1.0, -1.0)
        rc = L.gb300_conservation_noalloc(nx, ny, pad, fg.dptr(rho), fg.dptr(e),
                                          ctypes.cast(o, ctypes.POINTER(ctypes.c_double)))
        assert rc == 0, fg.lib().gb300_last_error_message()
        got.append((o[0], o[1]))
    return ref, got


def check_pair(ref, got):
    assert got[0] == got[1]  # same order of additions every call
    for g in got:
        np.testing.assert_allclose(g, ref, rtol=REL_TOL, atol=0)


def test_noalloc_matches_conservation_after_steps(fg):
    from flow_gb300 import problems
    rng = np.random.default_rng(7)
    prob = problems.Problem(301, 187, dt_param=1e-4).fields(
        1.0 + 0.5 * rng.random((187, 301)), 1.0 + rng.random((187, 301)))
    sim = fg.DeviceSim(prob.with_cfl_dt())
    sim.initial_timestep()
    sim.run(5)
    ref, got = totals_pair(fg, sim.nx, sim.ny, 2, sim.a["rho"], sim.a["e"], sim.a["reduce"])
    check_pair(ref, got)
    rho, e = sim.interior("rho"), sim.interior("e")
    np.testing.assert_allclose(got[0], (rho.sum(), (rho * e).sum()), rtol=REL_TOL)


def test_noalloc_two_meshes_in_a_row_and_row_limit(fg):
    """A square mesh, then a tall one at exactly the row limit (more rows than
    the kernel has warps, so rows are strided), with no state carried over."""
    import torch
    from flow_gb300 import problems
    sim = fg.DeviceSim(problems.sedov(512))
    sim.initial_timestep()
    sim.run(3)
    ref, got = totals_pair(fg, sim.nx, sim.ny, 2, sim.a["rho"], sim.a["e"], sim.a["reduce"])
    check_pair(ref, got)
    del sim
    nx, ny, pad = 12, MAX_ROWS + 4, 2
    g = torch.Generator(device="cpu").manual_seed(11)
    rho = (0.5 + torch.rand(ny * nx, generator=g, dtype=torch.float64)).cuda()
    e = (1.0 + torch.rand(ny * nx, generator=g, dtype=torch.float64)).cuda()
    reduce_array = torch.zeros(ny * nx, dtype=torch.float64, device="cuda")
    ref, got = totals_pair(fg, nx, ny, pad, rho, e, reduce_array)
    check_pair(ref, got)


def test_noalloc_rejects_more_rows_than_its_scratch(fg):
    import torch
    L = fg.lib()
    nx, ny, pad = 12, MAX_ROWS + 5, 2  # one interior row too many; arrays sized to match
    rho = torch.ones(ny * nx, dtype=torch.float64, device="cuda")
    e = torch.ones(ny * nx, dtype=torch.float64, device="cuda")
    out = (ctypes.c_double * 2)(-1.0, -1.0)
    outp = ctypes.cast(out, ctypes.POINTER(ctypes.c_double))
    L.gb300_clear_error()
    assert L.gb300_conservation_noalloc(nx, ny, pad, fg.dptr(rho), fg.dptr(e), outp) == GB300_ERR_ARG
    assert b"16384" in L.gb300_last_error_message()
    assert out[0] == -1.0
    L.gb300_clear_error()
    assert L.gb300_conservation_noalloc(nx, ny, pad, None, fg.dptr(e), outp) == GB300_ERR_ARG
    L.gb300_clear_error()
    # A valid call right after the rejections.
    assert L.gb300_conservation_noalloc(nx, ny - 1, pad, fg.dptr(rho), fg.dptr(e), outp) == 0
    assert out[0] == MAX_ROWS * (nx - 2 * pad) and out[1] == out[0]


def test_noalloc_on_a_non_default_stream(fg):
    """Both entry points routed to a caller's own stream (gb300_set_stream):
    two no-allocation calls in a row give the totals gb300_conservation gives
    on that stream.  The default stream is restored afterwards."""
    import torch
    from flow_gb300 import problems
    L = fg.lib()
    sim = fg.DeviceSim(problems.sedov(256))
    sim.initial_timestep()
    sim.run(4)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    try:
        assert L.gb300_set_stream(ctypes.c_void_p(stream.cuda_stream)) == 0
        ref, got = totals_pair(fg, sim.nx, sim.ny, 2, sim.a["rho"], sim.a["e"], sim.a["reduce"])
    finally:
        L.gb300_set_stream(None)
    check_pair(ref, got)
