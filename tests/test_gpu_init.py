"""Device-side problem set-up (gb300_fill_boxes, gb300_batch_fill_boxes)
against the host rasterisation of the same boxes (the rule the reference's
known answer pins: a cell takes the last box holding its left/bottom edge).
Bit-exact: the device evaluates the same comparisons on the same edges."""
import copy
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GB300_ERR_ARG = 2


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    return flow_gb300


def device_fill(fg, prob, boxes):
    import torch
    L = fg.lib()
    ex = torch.from_numpy(prob.edgex).cuda()
    ey = torch.from_numpy(prob.edgey).cuda()
    rho = torch.full((prob.ny * prob.nx,), -1.0, dtype=torch.float64, device="cuda")
    e = torch.full_like(rho, -1.0)
    assert L.gb300_fill_boxes(prob.nx, prob.ny, fg.dptr(ex), fg.dptr(ey), fg.boxes_array(boxes),
                              len(boxes), fg.dptr(rho), fg.dptr(e)) == 0
    torch.cuda.synchronize()
    return rho.cpu().numpy().reshape(prob.ny, prob.nx), e.cpu().numpy().reshape(prob.ny, prob.nx)


@pytest.mark.parametrize("shape", [(40, 40), (151, 93), (4096, 4096)])
def test_fill_boxes_matches_host_rasterisation(fg, shape):
    from flow_gb300.problems import Problem
    boxes = O.flow_params_boxes()
    prob = Problem(*shape).boxes(boxes)
    rho, e = device_fill(fg, prob, boxes)
    assert np.array_equal(rho, prob.rho) and np.array_equal(e, prob.e)
    if shape == (4096, 4096):
        # The known answer's box covers 819^2 cells (flow.tests:1).
        assert int((prob.interior(rho) == 1.0).sum()) == 819 * 819


def test_fill_boxes_two_region_and_blast(fg):
    from flow_gb300 import problems
    rng = np.random.default_rng(20261203)
    probs = [problems.two_region(n, rng) for n in (128, 192, 320, 1024)] + [problems.sedov(256)]
    for p in probs:
        rho, e = device_fill(fg, p, p.box_list)
        assert np.array_equal(rho, p.rho) and np.array_equal(e, p.e)


def test_fill_boxes_without_boxes_is_zero_and_rejects_too_many(fg):
    from flow_gb300.problems import Problem
    prob = Problem(16, 12)
    rho, e = device_fill(fg, prob, [])
    assert not rho.any() and not e.any()
    L = fg.lib()
    boxes = [(1.0, 1.0, 0.0, 0.0, 1.0, 1.0)] * 33
    import torch
    ex = torch.from_numpy(prob.edgex).cuda()
    ey = torch.from_numpy(prob.edgey).cuda()
    buf = torch.zeros(prob.nx * prob.ny, dtype=torch.float64, device="cuda")
    L.gb300_clear_error()
    assert L.gb300_fill_boxes(prob.nx, prob.ny, fg.dptr(ex), fg.dptr(ey), fg.boxes_array(boxes),
                              33, fg.dptr(buf), fg.dptr(buf)) == GB300_ERR_ARG
    L.gb300_clear_error()


def test_device_sim_fill_matches_upload(fg):
    from flow_gb300 import problems
    a = problems.sod(200, 136)
    b = copy.deepcopy(a)
    b.box_list = None  # host fields uploaded instead
    sa, sb = fg.DeviceSim(a), fg.DeviceSim(b)
    for s in (sa, sb):
        s.initial_timestep()
        s.run(5)
    for k in ("rho", "e", "u", "v", "rho_u", "rho_v"):
        assert np.array_equal(sa.host(k), sb.host(k)), k


def test_batch_fill_boxes_matches_host_state(fg):
    from flow_gb300 import problems
    rng = np.random.default_rng(7)
    probs = [problems.two_region(n, rng) for n in (128, 256, 192)]
    host = [copy.deepcopy(p) for p in probs]
    for p in host:
        p.box_list = None
    ba = fg.Batch(probs, precision=0)
    bb = fg.Batch(host, precision=0)
    ba.step(6)
    bb.step(6)
    for i in range(len(probs)):
        ra, ea, dta, _ = ba.state(i)
        rb, eb, dtb, _ = bb.state(i)
        assert np.array_equal(ra, rb) and np.array_equal(ea, eb) and tuple(dta) == tuple(dtb), i
