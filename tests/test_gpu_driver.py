"""The C host driver (flow.gb300, a restatement of the reference main.c over
the GPU arch layer and the kernel set) on the reference's own known-answer
case: flow.params at 4096^2 for 100 iterations must pass the reference's
validation against flow.tests (interior sums within 1e-5, main.c:144-212)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver():
    from flow_gb300 import build
    build.build()
    return build.DRIVER


def run_driver(driver, workdir, params_text=None, *options):
    """Runs the driver in workdir on the reference's flow.params, or on
    params_text saved as small.params (which flow.tests has no entry for)."""
    name = "flow.params" if params_text is None else "small.params"
    if params_text is None:
        shutil.copy(os.path.join(HERE, "golden", "flow.params"), workdir)
    else:
        with open(os.path.join(workdir, name), "w") as f:
            f.write(params_text)
    shutil.copy(os.path.join(HERE, "golden", "flow.tests"), workdir)
    out = subprocess.run([driver, name, "--quiet", *options], cwd=workdir, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout


def test_driver_passes_reference_known_answer(driver, tmp_path):
    out = run_driver(driver, str(tmp_path))
    assert "PASSED validation." in out, out
    got = re.search(r"Expected energy\s+([0-9.e+-]+), result was ([0-9.e+-]*[0-9])", out)
    assert got and abs(float(got.group(2)) / float(got.group(1)) - 1) < 1e-11, out


def test_driver_small_case_matches_oracle(driver, tmp_path):
    text = ("problem_0 density=0.125 energy=2.0 xpos=0.0 ypos=0.0 width=1.0 height=1.0\n"
            "problem_1 density=1.0 energy=2.5 xpos=0.25 ypos=0.5 width=0.5 height=0.25\n"
            "dt 1.0e-3\nnx 96\nny 80\niterations 30\nvisit_dump 0\n")
    out = run_driver(driver, str(tmp_path), text)
    m = re.search(r"density total ([0-9.e+-]+), energy total ([0-9.e+-]+)", out)
    assert m, out
    hm = O.HostMesh(96, 80, dt=1e-3)
    st = O.HostState(hm)
    O.fill_boxes(hm, st, [(0.125, 2.0, 0.0, 0.0, 1.0, 1.0), (1.0, 2.5, 0.25, 0.5, 0.5, 0.25)])
    O.initial_timestep(hm, st)
    O.run(hm, st, 30)
    assert abs(float(m.group(1)) - st.interior("rho").sum()) <= 1e-12 * st.interior("rho").sum()
    assert abs(float(m.group(2)) - st.interior("e").sum()) <= 1e-12 * st.interior("e").sum()
