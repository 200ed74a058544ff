"""The VisIt field dump of the GPU arch layer (write_all_ranks_to_visit,
called by the reference driver at main.c:108-114 and 129-135) through its C
ABI: it returns before the files exist, the timestep keeps running and
overwrites the density, and every dump must still hold the density of the
moment it was requested, as <name><tt>.dat (interior rows, little-endian
doubles) with a .bov header naming it."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def arch():
    import flow_gb300
    flow_gb300.lib()
    L = ctypes.CDLL(os.path.join(os.path.dirname(flow_gb300.LIB_PATH), "libflow_gb300_arch.so"))
    L.write_all_ranks_to_visit.argtypes = [ctypes.c_int] * 9 + [
        ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int,
        ctypes.c_double]
    L.write_all_ranks_to_visit.restype = None
    L.write_all_ranks_flush.argtypes = []
    L.write_all_ranks_flush.restype = None
    return L


def dump(arch, sim, name, tt, t):
    nb = (ctypes.c_int * 4)(-1, -1, -1, -1)
    arch.write_all_ranks_to_visit(sim.nx, sim.ny, sim.nx, sim.ny, 2, 0, 0, 0, 1, nb,
                                  sim.a["rho"].data_ptr(), name.encode(), tt, t)


def read_bov(path):
    out = {}
    with open(path) as f:
        for line in f:
            k, _, v = line.partition(":")
            out[k.strip()] = v.strip()
    return out


def test_dumps_hold_the_field_of_their_step(arch, tmp_path, monkeypatch):
    import flow_gb300 as fg
    from flow_gb300 import problems
    monkeypatch.chdir(tmp_path)
    fg.set_mode(fg.MODE_FUSED)
    sim = fg.DeviceSim(problems.sedov(200))
    sim.initial_timestep()
    snaps = {}
    t = 0.0
    for tt in range(7):
        sim.step()
        t += sim.mesh.dt
        if tt % 2 == 0:
            dump(arch, sim, "density", tt, t)  # returns at once; the steps go on
            snaps[tt] = (sim.interior("rho").copy(), t)
    arch.write_all_ranks_flush()
    for tt, (want, when) in snaps.items():
        data = np.fromfile(tmp_path / f"density{tt}.dat", dtype="<f8")
        assert data.size == want.size
        assert np.array_equal(data.reshape(want.shape), want), tt
        hdr = read_bov(tmp_path / f"density{tt}.bov")
        assert hdr["DATA_FILE"] == f"density{tt}.dat"
        assert hdr["DATA_SIZE"] == "200 200 1"
        assert hdr["DATA_FORMAT"] == "DOUBLE" and hdr["DATA_ENDIAN"] == "LITTLE"
        assert hdr["VARIABLE"] == "density"
        assert float(hdr["TIME"]) == pytest.approx(when, rel=1e-12)


def test_more_dumps_than_slots_in_a_row(arch, tmp_path, monkeypatch):
    """Five dumps back to back with no step between them and a ragged mesh:
    the later calls wait for free slots and every file is complete."""
    import flow_gb300 as fg
    from flow_gb300 import problems
    monkeypatch.chdir(tmp_path)
    sim = fg.DeviceSim(problems.sod(131, 77))
    sim.initial_timestep()
    sim.run(3)
    want = sim.interior("rho")
    for k in range(5):
        dump(arch, sim, "rho", k, 0.5 * k)
    arch.write_all_ranks_flush()
    for k in range(5):
        data = np.fromfile(tmp_path / f"rho{k}.dat", dtype="<f8").reshape(want.shape)
        assert np.array_equal(data, want), k
        assert read_bov(tmp_path / f"rho{k}.bov")["DATA_SIZE"] == "131 77 1"
