"""The C++ host driver (csrc/femgl_main.cc): it reads the reference's configuration file
format and keys, and on the GPU runs the Newton loop through the C ABI to the same answer
as the Python binding."""
import os
import re
import subprocess

import numpy as np
import pytest

from _lib import product

CONFIG = """# a small cube: 4^3 cells of side 1.25
subsection physical parameters
  set pressure in bar = 20.0   # bar
  set t_reduced = 0.6
  set trun on Strong Coupling Correction = true
end
subsection control parameters
  set cube half side length = 2.5
  set Number of initial global refinments = 2
  set Number of refinements = 0
  set Number of interations = 40
  set Cycle 0 linear solver tol = 1e-4
  set converge accuracy = 1e-10
end
"""


@pytest.fixture(scope="module")
def driver():
    pkg = product()
    path = os.path.join(os.path.dirname(pkg.build()), "femgl_gb300")
    assert os.path.exists(path)
    return path


def _write(tmp_path, text, name="configuration.prm"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_driver_reads_configuration(driver, tmp_path):
    out = subprocess.run([driver, _write(tmp_path, CONFIG), "--dry-run"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert "p = 20 bar, t = 0.6, SCC on, cube half side 2.5, 4^3 cells" in out.stdout
    assert "linear tol 0.0001, converge accuracy 1e-10" in out.stdout


PDW_SLAB = """# the periodic slab of the weak-coupling PDW scenario
subsection physical parameters
  set pressure in bar = 22.0
  set t_reduced = 0.5
  set amplitude u parameter = 0.8
end
subsection control parameters
  set half x length of retangle = 6.0
  set half y length of retangle = 4.0
  set half z length of retangle = 3.0
  set Number of initial global refinments = 3
end
"""


def test_driver_pdw_slab_scenario_reads_configuration(driver, tmp_path):
    out = subprocess.run([driver, _write(tmp_path, PDW_SLAB), "--scenario", "pdw-slab", "--dry-run"],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert "periodic slab 12 x 8 x 6 (x, y periodic), 8^3 cells, PDW start u = 0.8" in out.stdout
    # the declared defaults: half lengths 20, u = 1
    out = subprocess.run([driver, _write(tmp_path, "subsection physical parameters\nend\n"), "--scenario",
                          "pdw-slab", "--dry-run"], capture_output=True, text=True)
    assert out.returncode == 0 and "periodic slab 40 x 40 x 40 (x, y periodic), 16^3 cells, PDW start u = 1" in out.stdout
    bad = PDW_SLAB.replace("half y length of retangle = 4.0", "half y length of retangle = 0")
    r = subprocess.run([driver, _write(tmp_path, bad, "bad.prm"), "--scenario", "pdw-slab", "--dry-run"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "half lengths" in r.stderr
    r = subprocess.run([driver, _write(tmp_path, PDW_SLAB), "--scenario", "sphere", "--dry-run"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "unknown scenario" in r.stderr


def test_driver_defaults_and_errors(driver, tmp_path):
    # unset keys take the reference's declared defaults (cube half side 20, 2^4 cells)
    out = subprocess.run([driver, _write(tmp_path, "subsection physical parameters\nend\n"), "--dry-run"],
                         capture_output=True, text=True)
    assert out.returncode == 0 and "cube half side 20, 16^3 cells" in out.stdout
    assert "converge accuracy 5e-06" in out.stdout
    for bad in ("set x = 1\nend\n", "subsection a\n", "subsection a\n  set b\nend\n", "what\n"):
        r = subprocess.run([driver, _write(tmp_path, bad, "bad.prm"), "--dry-run"], capture_output=True, text=True)
        assert r.returncode == 2, bad
    r = subprocess.run([driver, str(tmp_path / "missing.prm"), "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 2 and "cannot open" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_driver_solves_like_the_binding(driver, tmp_path, precision):
    gl = product()
    out = subprocess.run([driver, _write(tmp_path, CONFIG), "--precision", precision, "--out",
                          str(tmp_path / "x.bin")], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    m = re.search(r"converged after (\d+) Newton iterations .*\|R\| = (\S+), F = (\S+),", out.stdout)
    assert m, out.stdout
    its, res, F = int(m.group(1)), float(m.group(2)), float(m.group(3))
    assert res <= 1e-10
    mesh = gl.cube_mesh(2.5, 4)
    prm = gl.Params.from_matep(20.0, 0.6, precision=gl.FP64 if precision == "fp64" else gl.MIXED,
                               precond=gl.PC_MULTIGRID)
    with gl.FemGL(mesh, prm) as f:
        f.set_solution(gl.bphase_guess(20.0, 0.6, mesh.nn))
        o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        x, Fb = f.solution(), f.free_energy()[0]
    assert its == int(o["newton_its"][0])
    assert abs(F - Fb) <= 1e-12 * abs(Fb)
    xd = np.fromfile(tmp_path / "x.bin", dtype=np.float64)
    assert np.array_equal(xd, x)


@pytest.mark.gpu
def test_driver_robin_faces_like_the_binding(driver, tmp_path):
    """The configuration's AdGR diffuse length turns on the Robin faces of the z boundary."""
    gl = product()
    cfg = CONFIG.replace("  set t_reduced = 0.6\n", "  set t_reduced = 0.6\n  set AdGR diffuse length = 2.0\n")
    out = subprocess.run([driver, _write(tmp_path, cfg), "--out", str(tmp_path / "x.bin")], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "Robin (AdGR) term" in out.stdout
    m = re.search(r"converged after (\d+) Newton iterations .*\|R\| = (\S+), F = (\S+),", out.stdout)
    assert m, out.stdout
    its, F = int(m.group(1)), float(m.group(3))
    mesh = gl.cube_mesh(2.5, 4)
    prm = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID, bt=2.0)
    with gl.FemGL(mesh, prm) as f:
        f.set_solution(gl.bphase_guess(20.0, 0.6, mesh.nn))
        o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        x, Fb = f.solution(), f.free_energy()[0]
    assert its == int(o["newton_its"][0])
    assert abs(F - Fb) <= 1e-12 * abs(Fb)
    assert np.array_equal(np.fromfile(tmp_path / "x.bin", dtype=np.float64), x)
    # and differs from the run without the face term
    prm0 = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    with gl.FemGL(mesh, prm0) as f:
        f.set_solution(gl.bphase_guess(20.0, 0.6, mesh.nn))
        f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        assert abs(f.free_energy()[0] - Fb) > 1e-6 * abs(Fb)


def test_driver_rejects_nonpositive_bt(driver, tmp_path):
    cfg = CONFIG.replace("  set t_reduced = 0.6\n", "  set t_reduced = 0.6\n  set AdGR diffuse length = 0\n")
    r = subprocess.run([driver, _write(tmp_path, cfg), "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 2 and "AdGR" in r.stderr


CYCLES = """subsection physical parameters
  set pressure in bar = 20.0
  set t_reduced = 0.6
end
subsection control parameters
  set cube half side length = 5.0
  set Number of initial global refinments = 2
  set Number of refinements = 2
  set Number of interations = 40
  set Cycle 0 refinement threshold = 1e6
  set Cycle 0 linear solver tol = 1e-3
  set Cycle 1 refinement threshold = 1e6
  set Cycle 1 do global refinement = true
  set Cycle 1 linear solver tol = 1e-3
  set Cycle 2 do global refinement = false
  set Cycle 2 linear solver tol = 1e-4
  set adaptive refinment ratio = 0.3
  set converge accuracy = 1e-10
end
"""


@pytest.mark.gpu
def test_driver_refinement_cycles_like_the_binding(driver, tmp_path):
    """run.cc's cycle loop: cycle 0 and 1 stall at once (threshold 1e6) and refine, globally
    then adaptively (GPU Kelly estimate, 30 % of the cells refined once), with the solution
    transferred each time; the same steps through the binding give the same answer."""
    gl = product()
    out = subprocess.run([driver, _write(tmp_path, CYCLES), "--out", str(tmp_path / "x.bin")], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "refinement cycle 1 (global): 512 cells" in out.stdout
    assert "refinement cycle 2 (adaptive)" in out.stdout
    m_its = re.search(r"converged after (\d+) Newton iterations .*\|R\| = (\S+), F = (\S+),", out.stdout)
    assert m_its, out.stdout
    F_drv = float(m_its.group(3))

    lo, hi = [-5.0] * 3, [5.0] * 3
    prm = gl.Params.from_matep(20.0, 0.6, precision=gl.MIXED, precond=gl.PC_MULTIGRID)
    m0 = gl.cube_mesh(5.0, 4)
    with gl.FemGL(m0, prm) as f:
        f.set_solution(gl.bphase_guess(20.0, 0.6, m0.nn))
        f.assemble_system()
        f.solve(1e-3, allow_unconverged=True)
        f.newton_iteration()
        x0 = f.solution()
    m1 = gl.cube_mesh(5.0, 8)
    with gl.FemGL(m1, prm) as f:
        f.set_solution(gl.box_interpolate(lo, hi, (4, 4, 4), x0, m1.xyz))
        f.assemble_system()
        f.solve(1e-3, allow_unconverged=True)
        f.newton_iteration()
        x1 = f.solution()
        f.estimate_error()
        flags = f.refine_flags(0.3)
    m2 = gl.box_mesh_refine(lo, hi, (8, 8, 8), flags)
    assert f"refinement cycle 2 (adaptive): {m2.nc} cells" in out.stdout
    with gl.FemGL(m2, prm) as f:
        f.set_solution(gl.box_interpolate(lo, hi, (8, 8, 8), x1, m2.xyz))
        o = f.run(max_newton=40, linear_tol=1e-4, converge_acc=1e-10)
        x, F = f.solution(), f.free_energy()[0]
    assert o["converged"]
    assert abs(F_drv - F) <= 1e-12 * abs(F)
    assert np.array_equal(np.fromfile(tmp_path / "x.bin", dtype=np.float64), x)
