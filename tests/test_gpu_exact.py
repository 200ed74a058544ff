"""GPU parity of the stage entry points (omp3/flow.h:4-88) and of the exact
timestep mode, through the C ABI, against the oracle.

stages.cu evaluates every expression in the reference's order without
floating-point contraction, so the bar here is bit-exact equality (NaN
patterns included) with the C restatement and with the golden fixtures that
the reference produced.
"""
import ctypes
import glob
import os
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    flow_gb300.set_mode(flow_gb300.MODE_EXACT)
    yield flow_gb300
    flow_gb300.set_mode(flow_gb300.MODE_FUSED)


def make_pair(fg, rho0, e0, dt_param):
    """The same initial state on the device and in the oracle."""
    from flow_gb300.problems import Problem
    gny, gnx = rho0.shape
    prob = Problem(gnx, gny, dt_param=dt_param).fields(rho0, e0)
    sim = fg.DeviceSim(prob)
    hm = O.HostMesh(gnx, gny, dt=dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, rho0, e0)
    return sim, hm, st


def assert_state_equal(sim, st, fields=None, exact=True):
    for k in fields or O.FIELDS:
        if k == "reduce":
            continue
        got = sim.host(k)
        if exact:
            assert np.array_equal(got, st[k], equal_nan=True), k
        else:
            np.testing.assert_allclose(got, st[k], rtol=1e-13, atol=0, err_msg=k)


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_exact_mode_reproduces_reference_fixture(fg, path):
    from flow_gb300.problems import Problem
    z = np.load(path)
    gny, gnx = z["rho0"].shape
    sim = fg.DeviceSim(Problem(gnx, gny, dt_param=float(z["dt_param"])).fields(z["rho0"], z["e0"]))
    sim.initial_timestep()
    hist = [(sim.mesh.dt, sim.mesh.dt_h)]
    for _ in range(int(z["steps"])):
        sim.step()
        hist.append((sim.mesh.dt, sim.mesh.dt_h))
    assert np.array_equal(np.array(hist), z["dt_hist"])
    for k in O.FIELDS:
        if k != "reduce":
            assert np.array_equal(sim.host(k), z[f"out_{k}"], equal_nan=True), k


def test_exact_mode_sod_512_100_steps(fg):
    """Config 0 of the benchmark set: 512^2 Sod tube, 100 iterations, FP64,
    per-cell comparison with the oracle (bit-exact in this mode)."""
    from flow_gb300 import problems
    prob = problems.sod(512)
    sim, hm, st = make_pair(fg, prob.interior(prob.rho).copy(), prob.interior(prob.e).copy(), prob.dt_param)
    sim.initial_timestep()
    O.initial_timestep(hm, st)
    assert sim.mesh.dt == hm.mesh.dt
    for tt in range(100):
        sim.step()
        O.step(hm, st, tt)
        assert sim.mesh.dt == hm.mesh.dt and sim.mesh.dt_h == hm.mesh.dt_h, tt
    assert_state_equal(sim, st)


def _random_state(rng, sim, st):
    """Identical random arrays in every field on both sides."""
    import torch
    for k in O.FIELDS:
        if k == "reduce":
            continue
        n = st[k].size
        if k in ("rho", "rho_old"):
            a = rng.uniform(0.3, 2.0, n)
        elif k in ("e", "P"):
            a = rng.uniform(0.2, 3.0, n)
        elif k in ("Qxx", "Qyy"):
            a = rng.uniform(0.0, 1.0, n)            # the viscous stress is never negative
        else:
            a = rng.uniform(-1.0, 1.0, n)
            a[rng.random(n) < 0.05] = 0.0          # exact zeros exercise the limiter branches
        st[k][:] = a
        sim.a[k].copy_(torch.from_numpy(a))


STAGES = ["equation_of_state", "pressure_acceleration", "artificial_viscosity",
          "shock_heating_and_work", "advect_mass_and_energy_even",
          "advect_mass_and_energy_odd", "x_mass_and_energy_flux", "y_mass_and_energy_flux",
          "advect_momentum_even", "advect_momentum_odd", "momentum_x_flux_in_x",
          "momentum_x_flux_in_y", "momentum_y_flux_in_x", "momentum_y_flux_in_y"]


@pytest.mark.parametrize("stage", STAGES)
@pytest.mark.parametrize("shape", [(17, 13), (64, 40)])
def test_stage_entry_point_bit_exact(fg, stage, shape):
    rng = np.random.default_rng(zlib.crc32(f"{stage}{shape}".encode()))
    gnx, gny = shape
    sim, hm, st = make_pair(fg, np.ones((gny, gnx)), np.ones((gny, gnx)), 1e-3)
    _random_state(rng, sim, st)
    L, R = fg.lib(), O.lib("port")
    d = {k: fg.dptr(sim.a[k]) for k in O.FIELDS}
    h = {k: O.ptr(st[k]) for k in O.FIELDS}
    dm, hmp = ctypes.byref(sim.mesh), ctypes.byref(hm.mesh)
    nx, ny = hm.nx, hm.ny
    dt, dt_h = 1.3e-3, 1.1e-3

    def both(fn):
        fn(L, d, dm, sim.mesh)
        fn(R, h, hmp, hm.mesh)

    if stage == "equation_of_state":
        both(lambda X, a, mp, m: X.equation_of_state(nx, ny, a["P"], a["rho"], a["e"]))
    elif stage == "pressure_acceleration":
        both(lambda X, a, mp, m: X.pressure_acceleration(nx, ny, mp, dt, a["rho_u"], a["rho_v"], a["u"], a["v"], a["P"], a["rho"], m.edgedx, m.edgedy, m.celldx, m.celldy))
    elif stage == "artificial_viscosity":
        both(lambda X, a, mp, m: X.artificial_viscosity(nx, ny, mp, dt, a["Qxx"], a["Qyy"], a["u"], a["v"], a["rho_u"], a["rho_v"], a["rho"], m.edgedx, m.edgedy, m.celldx, m.celldy))
    elif stage == "shock_heating_and_work":
        both(lambda X, a, mp, m: X.shock_heating_and_work(nx, ny, mp, dt_h, a["e"], a["P"], a["u"], a["v"], a["rho"], a["Qxx"], a["Qyy"], m.celldx, m.celldy))
    elif stage.startswith("advect_mass_and_energy"):
        tt = 0 if stage.endswith("even") else 1
        both(lambda X, a, mp, m: X.advect_mass_and_energy(nx, ny, mp, tt, dt, dt_h, a["rho"], a["e"], a["rho_old"], a["F_x"], a["F_y"], a["uF_x"], a["uF_y"], a["u"], a["v"], m.edgedx, m.edgedy, m.celldx, m.celldy))
    elif stage == "x_mass_and_energy_flux":
        both(lambda X, a, mp, m: X.x_mass_and_energy_flux(nx, ny, 1, mp, dt, dt_h, a["rho"], a["rho_old"], a["e"], a["u"], a["F_x"], a["uF_x"], m.celldx, m.edgedx, m.celldy, m.edgedy))
    elif stage == "y_mass_and_energy_flux":
        both(lambda X, a, mp, m: X.y_mass_and_energy_flux(nx, ny, 0, mp, dt, dt_h, a["rho"], a["rho_old"], a["e"], a["v"], a["F_y"], a["uF_y"], m.celldx, m.edgedx, m.celldy, m.edgedy))
    elif stage.startswith("advect_momentum"):
        tt = 0 if stage.endswith("even") else 1
        both(lambda X, a, mp, m: X.advect_momentum(nx, ny, tt, mp, dt_h, dt, a["u"], a["v"], a["uF_x"], a["uF_y"], a["vF_x"], a["vF_y"], a["rho_u"], a["rho_v"], a["rho"], a["F_x"], a["F_y"], m.edgedx, m.edgedy, m.celldx, m.celldy))
    elif stage == "momentum_x_flux_in_x":
        both(lambda X, a, mp, m: X.momentum_x_flux_in_x(nx, ny, mp, dt_h, a["u"], a["uF_x"], a["F_x"], m.edgedx, m.edgedy, m.celldx))
    elif stage == "momentum_x_flux_in_y":
        both(lambda X, a, mp, m: X.momentum_x_flux_in_y(nx, ny, mp, dt_h, a["u"], a["v"], a["uF_y"], a["F_y"], m.edgedx, m.edgedy, m.celldy))
    elif stage == "momentum_y_flux_in_x":
        both(lambda X, a, mp, m: X.momentum_y_flux_in_x(nx, ny, mp, dt_h, a["u"], a["v"], a["vF_x"], a["F_x"], m.edgedx, m.celldy, m.celldx))
    elif stage == "momentum_y_flux_in_y":
        both(lambda X, a, mp, m: X.momentum_y_flux_in_y(nx, ny, mp, dt_h, a["v"], a["vF_y"], a["F_y"], m.edgedy, m.celldx, m.celldy))
    fg.check()
    assert_state_equal(sim, st)


def test_set_timestep_bit_exact(fg):
    rng = np.random.default_rng(7)
    sim, hm, st = make_pair(fg, rng.uniform(0.5, 2, (30, 41)), rng.uniform(0.5, 2, (30, 41)), 1e-3)
    _random_state(rng, sim, st)
    for first in (0, 1):
        sim.mesh.dt = hm.mesh.dt = 2.5e-3
        sim.mesh.dt_h = hm.mesh.dt_h = 2.0e-3
        fg.lib().set_timestep(hm.nx, hm.ny, fg.dptr(sim.a["Qxx"]), fg.dptr(sim.a["Qyy"]), fg.dptr(sim.a["rho"]), fg.dptr(sim.a["e"]), ctypes.byref(sim.mesh), fg.dptr(sim.a["reduce"]), first, sim.mesh.celldx, sim.mesh.celldy)
        fg.check()
        O.lib().set_timestep(hm.nx, hm.ny, O.ptr(st["Qxx"]), O.ptr(st["Qyy"]), O.ptr(st["rho"]), O.ptr(st["e"]), ctypes.byref(hm.mesh), O.ptr(st["reduce"]), first, hm.mesh.celldx, hm.mesh.celldy)
        assert (sim.mesh.dt, sim.mesh.dt_h) == (hm.mesh.dt, hm.mesh.dt_h)


def test_conservation_totals(fg):
    rng = np.random.default_rng(3)
    r, e = rng.uniform(0.1, 2, (257, 129)), rng.uniform(0.1, 5, (257, 129))
    sim, hm, st = make_pair(fg, r, e, 1e-3)
    got = sim.conservation()
    want = O.conservation(hm, st)
    np.testing.assert_allclose(got, want, rtol=1e-13)


@pytest.mark.parametrize("width", [1024 + 256 + 7, 2048, 300])
def test_conservation_totals_runs_of_equal_cells(fg, width):
    """Rows wide enough for the full 1024-column chunks, the single 256-column
    groups and the ragged tail, with runs of equal (rho, e) groups broken by
    a blast, a changed background and a lone perturbed cell."""
    rng = np.random.default_rng(4)
    ny = 37
    r, e = np.ones((ny, width)), np.full((ny, width), 1e-5)
    r[10:14, 40:300] = rng.uniform(0.5, 2.0, (4, 260))
    e[10:14, 40:300] = rng.uniform(1.0, 9.0, (4, 260))
    r[20:, :] = 1.25  # a second run of equal groups
    e[25, width // 2] = 3.0  # one cell breaks its group
    sim, hm, st = make_pair(fg, r, e, 1e-3)
    got = sim.conservation()
    want = O.conservation(hm, st)
    np.testing.assert_allclose(got, want, rtol=1e-13)


def test_boundary_fill_bit_exact(fg):
    rng = np.random.default_rng(11)
    sim, hm, st = make_pair(fg, np.ones((9, 14)), np.ones((9, 14)), 1e-3)
    _random_state(rng, sim, st)
    for (k, w, hgt, inv) in [("rho", hm.nx, hm.ny, 0), ("u", hm.nx + 1, hm.ny, 1),
                             ("v", hm.nx, hm.ny + 1, 2), ("uF_y", hm.nx + 1, hm.ny + 1, 0)]:
        fg.lib().handle_boundary_2d(w, hgt, ctypes.byref(sim.mesh), fg.dptr(sim.a[k]), inv, 1)
        O.lib().handle_boundary_2d(w, hgt, ctypes.byref(hm.mesh), O.ptr(st[k]), inv, 1)
    fg.check()
    assert_state_equal(sim, st)


def test_rejects_unsupported_sizes(fg):
    """Too-small meshes are refused on the host with GB300_ERR_ARG."""
    sim, hm, st = make_pair(fg, np.ones((4, 4)), np.ones((4, 4)), 1e-3)
    sim.mesh.local_nx = 5  # one interior cell
    st_code = fg.lib().gb300_solve_hydro_2d(ctypes.byref(sim.mesh), 0, *sim.args())
    assert st_code == 2
    with pytest.raises(fg.FlowError):
        fg.check()
    sim.mesh.local_nx = hm.nx
    sim.mesh.neighbours[1] = 3  # a neighbouring rank: halo exchange is out of scope
    assert fg.lib().gb300_solve_hydro_2d(ctypes.byref(sim.mesh), 0, *sim.args()) == 2
    fg.lib().gb300_clear_error()
