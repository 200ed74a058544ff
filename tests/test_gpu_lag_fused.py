"""The one-kernel Lagrangian phase (GB300_MODE_FUSED_LAG) against the same
step with the Lagrangian phase as four kernels (GB300_MODE_FUSED): both are
built from the same expressions in the same order, so every state array and
dt must be equal bit for bit after every step, on power-of-two and general
meshes, ragged sizes, problems with walls hit by the flow, and every tile
height.  The four-kernel form is itself held to the oracle by
test_gpu_fused.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    yield flow_gb300
    flow_gb300.set_mode(flow_gb300.MODE_FUSED)
    flow_gb300.lib().gb300_set_lagrangian_rows(32)


def _problems():
    from flow_gb300 import problems
    rng = np.random.default_rng(7)
    return {
        "sod_96x80": problems.sod(96, 80),                 # spacings 1/96: general mesh
        "sedov_128": problems.sedov(128),
        "two_region_151": problems.two_region(151, rng),   # odd side
        "smooth_130": problems.smooth_random(130, rng),    # in motion everywhere
        "reference_box_200": problems.reference_problem(200).with_cfl_dt(),
    }


def run_pair(fg, prob, steps, rows):
    L = fg.lib()
    sims = {}
    for mode in (fg.MODE_FUSED, fg.MODE_FUSED_LAG):
        fg.set_mode(mode)
        sims[mode] = fg.DeviceSim(prob)
        sims[mode].initial_timestep()
    assert L.gb300_set_lagrangian_rows(rows) == 0
    for tt in range(steps):
        for mode, sim in sims.items():
            fg.set_mode(mode)
            sim.step()
        a, b = sims[fg.MODE_FUSED], sims[fg.MODE_FUSED_LAG]
        assert a.mesh.dt == b.mesh.dt and a.mesh.dt_h == b.mesh.dt_h, tt
        if tt % 5 == 4 or tt == steps - 1:
            for k in STATE:
                x, y = a.interior(k), b.interior(k)
                same = np.array_equal(x.view(np.uint64), y.view(np.uint64))
                assert same, (tt, k, int(np.count_nonzero(x != y)))
    fg.set_mode(fg.MODE_FUSED)


@pytest.mark.parametrize("name", list(_problems()))
def test_lagrangian_kernel_bit_identical(fg, name):
    run_pair(fg, _problems()[name], steps=20, rows=32)


@pytest.mark.parametrize("rows", [1, 5, 16, 64])
def test_lagrangian_kernel_tile_heights(fg, rows):
    from flow_gb300 import problems
    run_pair(fg, problems.sod(150, 90), steps=10, rows=rows)


def test_lagrangian_kernel_blast_4096(fg):
    """The benchmark mesh, a few steps (most of it at rest)."""
    from flow_gb300 import problems
    run_pair(fg, problems.sedov(4096), steps=6, rows=32)
