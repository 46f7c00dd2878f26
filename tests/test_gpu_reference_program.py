"""The reference's own host program on a lattice, with libgfx as its CUDA side.

oracle/ref_link_main.c runs the reference main's flow (cudagaugefix.cu:599-828) over
the reference's host C files, unchanged -- read_input.c parses the input file,
gauge_io.c reads and writes the ILDG files, su3manip.c makes the random start,
observables.c forms g U g^+ on the host -- and calls init_gaugefixing, init_MT,
simannealing_gauge, overrelax_gauge and calc_plaquette in libgfx.so.  It runs here
on an 8^4 configuration next to this repository's own program
(cudagfx_gb300/host/gfx_gaugefix.c) on the same input file, twister seed and ILDG
file.  The two must print the same check lines (the same solve), write the same
LIME record layout and ILDG metadata byte for byte, and gauge-fixed fields that agree
to FP64 rounding (the reference forms g U g^+ on the host, gfx_gaugefix on the
device)."""
import os
import struct
import subprocess

import numpy as np
import pytest

import cudagfx_gb300 as gfx
from cudagfx_gb300 import build as gbuild
from conftest import smooth_links

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 8)

INPUT = """# input file for GPU gauge fixing
T=8
L=8

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


def _lime_records(path):
    """(type, data) of every LIME record: 144-byte header (magic, version, flags, data
    length, 128-byte type), data padded to 8 bytes"""
    out = []
    raw = open(path, "rb").read()
    pos = 0
    while pos < len(raw):
        magic, _, _, n = struct.unpack(">IHHQ", raw[pos:pos + 16])
        assert magic == 0x456789AB
        rtype = raw[pos + 16:pos + 144].rstrip(b"\0").decode()
        data = raw[pos + 144:pos + 144 + n]
        out.append((rtype, data))
        pos += 144 + ((n + 7) // 8) * 8
    return out


def test_reference_host_program_on_libgfx_matches_gfx_gaugefix(tmp_path, oracle, mt_params):
    from oracle import build as ob
    prog = ob.build_reference_link()
    if not prog:
        pytest.skip("copies of the reference's host files are not present")
    gbuild.build()
    u = smooth_links(DIMS, 0.45, 71)
    gfx.ildg_write(str(tmp_path / "conf.ildg"), DIMS, u, 64, 0.0, 6.0)
    (tmp_path / "input.in").write_text(INPUT)
    dat = tmp_path / "MersenneTwister.dat"
    np.asarray(mt_params, dtype="<u4").tofile(dat)
    env = dict(os.environ, GFX_MT_DAT=str(dat), GFX_MT_SEED="1234")
    ref = subprocess.run([prog, "input.in", "conf.ildg"], capture_output=True, text=True,
                         cwd=tmp_path, env=env, timeout=300)
    assert ref.returncode == 0, ref.stdout[-2000:] + ref.stderr[-2000:]
    own = subprocess.run([gbuild.PROGRAM, "-i", "input.in", "-f", "conf.ildg", "-m", "1234",
                          "-o", "gfx_conf.ildg"], capture_output=True, text=True,
                         cwd=tmp_path, env=env, timeout=300)
    assert own.returncode == 0, own.stdout[-2000:] + own.stderr[-2000:]

    def checks(out):
        return [ln for ln in out.splitlines() if ln.startswith("iter ")]

    assert "CONVERGENCE" in ref.stdout and len(checks(ref.stdout)) > 3
    assert checks(ref.stdout) == checks(own.stdout)  # the same annealing and solve

    a, b = tmp_path / "landau_conf.ildg", tmp_path / "gfx_conf.ildg"
    ra, rb = _lime_records(a), _lime_records(b)
    assert [(t, len(d)) for t, d in ra] == [(t, len(d)) for t, d in rb]
    for (t, da), (_, db) in zip(ra, rb):
        if t != "ildg-binary-data":
            assert da == db, t  # ildg-format and xlf-info byte for byte
    fa, _ = gfx.ildg_read(str(a), DIMS)
    fb, _ = gfx.ildg_read(str(b), DIMS)
    assert np.max(np.abs(fa - fb)) < 1e-13
    lat = oracle.lattice(DIMS)
    _, mx = oracle.dAdA18(lat, fa.reshape(-1, 18))
    assert mx < 1e-11 * 1.01  # the ORX criterion on the reference's own output
    assert oracle.mean_plaq18(lat, fa.reshape(-1, 18)) == pytest.approx(
        oracle.mean_plaq18(lat, np.asarray(u).reshape(-1, 18)), rel=1e-12)
