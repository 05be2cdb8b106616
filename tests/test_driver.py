"""The drop-in driver executable (the reference's main: parameter file with globals.h names,
fields/%c.%07d.bin output, restart, solution.txt)."""
import os
import subprocess

import numpy as np
import pytest

from cudanavierstokes_gb300 import build
from cudanavierstokes_gb300.initial import read_fields, tgv_reference_fields
from cudanavierstokes_gb300.params import tgv_params
from cudanavierstokes_gb300.solver import host_grid

PARAMS = """# Taylor-Green box, reference parameter names
mx_tot = 16
my_tot = 20
mz_tot = 24
Lx = 6.283185307179586
Ly = 6.283185307179586
Lz = 6.283185307179586
stencilSize = 4
stencilVisc = 4
nsteps = {nsteps}
nfiles = {nfiles}
restartFile = {restart}
CFL = 0.5
Re = 1600.0
Pr = 0.71
Ma = 0.1
viscexp = 1.0
gam = 1.4
checkCFLcondition = 100
checkBulk = 2
"""


def _run(tmp_path, nsteps=4, nfiles=2, restart=-1):
    build.build()
    pf = tmp_path / "params.txt"
    pf.write_text(PARAMS.format(nsteps=nsteps, nfiles=nfiles, restart=restart))
    return subprocess.run([build.DRIVER, str(pf), str(tmp_path)], capture_output=True, text=True, timeout=600)


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_driver_fails_loudly_without_gpu(tmp_path):
    if _gpu_available():
        pytest.skip("a GPU is present")
    r = _run(tmp_path)
    assert r.returncode == 2 and "no CUDA device" in r.stderr
    p = tgv_params(16).copy(my=20, mz=24)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "fields" / "x.bin"), host_grid(p)["x"])


@pytest.mark.gpu
def test_driver_matches_library_and_restarts(tmp_path, gpu_lib):
    from cudanavierstokes_gb300 import Solver
    r = _run(tmp_path, nsteps=4, nfiles=2)
    assert r.returncode == 0, r.stderr
    p = tgv_params(16).copy(my=20, mz=24, check_bulk=2)
    out2 = read_fields(str(tmp_path / "fields"), 2, p.shape)
    # file 0 is the initial field; the driver evaluates sin/cos with the C library and
    # numpy may use its own vectorised versions, which can differ in the last bit
    out0 = read_fields(str(tmp_path / "fields"), 0, p.shape)
    for a, b in zip(out0, tgv_reference_fields(p)):
        np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14)
    s = Solver(p)
    s.copy_field_in(*out0)
    s.run(4)
    s.run(4)
    for a, b in zip(out2, s.copy_field_out()):
        np.testing.assert_array_equal(a, b)
    assert (tmp_path / "solution.txt").read_text().strip()
    # prof.txt: the plane profiles of the last file, as the reference writes them
    prof = np.loadtxt(tmp_path / "prof.txt")
    np.testing.assert_allclose(prof, s.plane_stats().T, rtol=0, atol=5.01e-7)
    assert "friction Reynolds number" in r.stdout
    # XDMF descriptor: one uniform grid per written file, attributes pointing at them
    import xml.etree.ElementTree as ET
    root = ET.parse(tmp_path / "fields" / "fields.xmf").getroot()
    grids = root.findall("./Domain/Grid/Grid")
    assert [g.get("Name") for g in grids] == ["T0000000", "T0000001", "T0000002"]
    for g in grids:
        for att in g.findall("Attribute"):
            fn = att.find("DataItem").text.strip()
            assert (tmp_path / "fields" / fn).is_file()
            assert att.find("DataItem").get("Dimensions").split() == ["24", "20", "16"]
    times = [float(v) for v in root.find("./Domain/Grid/Time/DataItem").text.split()]
    assert times[0] == 0.0 and times[1] < times[2]
    # restart from file 1 for one file reproduces file 2
    out_dir = tmp_path / "restart"
    (out_dir / "fields").mkdir(parents=True)
    for c in "ruvwe":
        os.link(tmp_path / "fields" / f"{c}.0000001.bin", out_dir / "fields" / f"{c}.0000001.bin")
    os.link(tmp_path / "fields" / "scalars.0000001.txt", out_dir / "fields" / "scalars.0000001.txt")
    r = _run(out_dir, nsteps=4, nfiles=1, restart=1)
    assert r.returncode == 0, r.stderr
    for a, b in zip(read_fields(str(out_dir / "fields"), 2, p.shape), out2):
        np.testing.assert_array_equal(a, b)
    # the restart continues the clock from the saved scalars
    t_full = (tmp_path / "fields" / "scalars.0000002.txt").read_text()
    assert (out_dir / "fields" / "scalars.0000002.txt").read_text() == t_full


BL_PARAMS = """# boundary layer from generated self-similar inflow profiles
mx_tot = 16
my_tot = 8
mz_tot = 160
Lx = 20.0
Ly = 7.0
Lz = 100.0
stencilSize = 3
stencilVisc = 2
nsteps = 3
nfiles = 1
restartFile = -1
CFL = 0.75
Re = 1500.0
Pr = 0.75
Ma = 0.35
viscexp = 1.5
gam = 1.4
boundaryLayer = 1
perturbed = 1
periodicX = 0
nonUniformX = 1
stretch = 5.0
checkCFLcondition = 1
checkBulk = 1
"""


@pytest.mark.gpu
def test_driver_boundary_layer_from_generated_profiles(tmp_path, gpu_lib, oracle_mod):
    """The driver's boundary-layer start (sponge references from blasius1D/*.bin, which
    cudanavierstokes_gb300.blasius writes) and three steps, against the oracle."""
    pytest.importorskip("scipy")
    from cudanavierstokes_gb300.blasius import self_similar_profiles, write_profiles
    from cudanavierstokes_gb300.params import boundary_layer_params
    from tests._util import state_errors
    build.build()
    p = boundary_layer_params(16, 8, 160).copy(check_cfl=1, check_bulk=1)   # as the parameter file
    prof = self_similar_profiles(p.gam, p.Ma, p.Pr)
    write_profiles(str(tmp_path), prof)
    pf = tmp_path / "params.txt"
    pf.write_text(BL_PARAMS)
    r = subprocess.run([build.DRIVER, str(pf), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    o = oracle_mod.Oracle(p)
    spx, spz = o.sponge_strengths()
    args = [prof[k] for k in ("x", "r", "u", "w", "e")]
    rref, uref, wref, eref = o.sponge_refs(*args)
    o.set_sponge(spx, spz, rref, uref, wref, eref)
    o.set_state(*[np.broadcast_to(a[:, None, :], p.shape).copy() for a in (rref, uref, np.zeros_like(rref), wref, eref)])
    np.testing.assert_array_equal(read_fields(str(tmp_path / "fields"), 0, p.shape)[0], o.get_state()[0])
    o.run(3)
    assert max(state_errors(read_fields(str(tmp_path / "fields"), 1, p.shape), o.get_state())) <= 1e-12
