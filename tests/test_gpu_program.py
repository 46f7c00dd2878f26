"""The gauge-fixing program (cudagfx_gb300/host/gfx_gaugefix.c): the reference main's
flow -- input file, ILDG configuration in, annealing and overrelaxation through the
reference-named entry points, gauge-fixed ILDG field out -- with its exit codes."""
import os
import subprocess

import numpy as np
import pytest

import cudagfx_gb300 as gfx
from cudagfx_gb300 import build as gbuild
from conftest import smooth_links

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 8)

INPUT = """# input file for GPU gauge fixing
T=8
L=4

RandSeed = 351

BeginSAInit
  Tmin = 1.0e-2
  Tmax = 0.5
  ckinterval = 50
  Nstep = 100
  expo = -1.0
EndSAInit

BeginORXInit
  eps = 1.0e-11
  ckinterval = 20
  maxit = 5000
EndORXInit
"""


def _run(tmp_path, mt_params, *args):
    dat = tmp_path / "MersenneTwister.dat"
    if not dat.exists():
        np.asarray(mt_params, dtype="<u4").tofile(dat)
    env = dict(os.environ, GFX_MT_DAT=str(dat))
    return subprocess.run([gbuild.PROGRAM] + list(args), capture_output=True, text=True,
                          cwd=tmp_path, env=env, timeout=300)


@pytest.fixture
def config(tmp_path):
    u = smooth_links(DIMS, 0.5, 31)
    p = tmp_path / "conf.ildg"
    gfx.ildg_write(str(p), DIMS, u, 64, 0.0, 6.0)
    (tmp_path / "input.in").write_text(INPUT)
    return p, u


def test_program_fixes_and_writes(tmp_path, config, oracle, mt_params):
    p, u = config
    r = _run(tmp_path, mt_params, "-i", "input.in", "-f", "conf.ildg", "-p", "mixed", "-m", "1234")
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Starting simulated annealing" in r.stdout and "CONVERGENCE" in r.stdout
    out = tmp_path / "landau_conf.ildg"
    fixed, info = gfx.ildg_read(str(out), DIMS)
    assert info["beta"] == pytest.approx(6.0)
    lat = oracle.lattice(DIMS)
    dada, mx = oracle.dAdA18(lat, fixed.reshape(-1, 18))
    assert mx < 1e-11 * 1.01  # the ORX criterion (maxdAdA, as in overrelax.cu:794)
    assert oracle.mean_plaq18(lat, fixed.reshape(-1, 18)) == pytest.approx(
        oracle.mean_plaq18(lat, np.asarray(u).reshape(-1, 18)), rel=1e-12)
    # the output file exists now: the reference refuses to overwrite it (exit(-1))
    r2 = _run(tmp_path, mt_params, "-i", "input.in", "-f", "conf.ildg")
    assert r2.returncode == 255 and "is present" in r2.stdout


def test_program_thermalizes(tmp_path, config, mt_params):
    (tmp_path / "therm.in").write_text(
        "T=8\nL=4\nRandSeed = 7\nBeginTHERMInit\n  Nsweep = 10\n  beta = 6.0\n"
        "  ckinterval = 5\n  start = cold\nEndTHERMInit\n")
    r = _run(tmp_path, mt_params, "-i", "therm.in", "-f", "conf.ildg", "-m", "99")
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    u, info = gfx.ildg_read(str(tmp_path / "thermalized_conf.ildg"), DIMS)
    assert 0.3 < info["plaquette"] < 0.99  # moved away from the cold start


def test_program_errors(tmp_path, config, mt_params):
    r = _run(tmp_path, mt_params, "-i", "input.in", "-f", "missing.ildg")
    assert r.returncode == 1 and "Error reading configuration" in r.stdout
    (tmp_path / "bad.in").write_text("T=8\nL=4\nnonsense here\n")
    r = _run(tmp_path, mt_params, "-i", "bad.in", "-f", "conf.ildg")
    assert r.returncode == 2 and "Parsing error in line 3" in r.stdout
    (tmp_path / "wrong.in").write_text(INPUT.replace("L=4", "L=6"))
    r = _run(tmp_path, mt_params, "-i", "wrong.in", "-f", "conf.ildg")
    assert r.returncode == 1
    (tmp_path / "hard.in").write_text(INPUT.replace("maxit = 5000", "maxit = 20")
                                      .replace("Nstep = 100", "Nstep = 2"))
    r = _run(tmp_path, mt_params, "-i", "hard.in", "-f", "conf.ildg", "-o", "x.ildg")
    # exit(300) as in the reference; a process status keeps the low 8 bits
    assert r.returncode == 300 % 256 and "Gauge condition not reached" in r.stdout
