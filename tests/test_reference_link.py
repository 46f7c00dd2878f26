"""The drop-in boundary at link level: the reference's own host C files
(read_input.c, gauge_io.c, spinor_io.c, cksum.c, su3manip.c, observables.c, rngs.c,
complex.c), compiled unchanged with oracle/ref_link_main.c (the reference main's
host-side flow), link against libgfx.so, which supplies every CUDA-side entry
point, device global and LIME function they call.  CPU only: the program is
linked and started (usage path), not run on a lattice.  Skipped where the
reference sources are absent."""
import ctypes
import subprocess

import pytest

import cudagfx_gb300 as gfx


def test_reference_host_files_link_against_libgfx():
    from oracle import build as ob
    prog = ob.build_reference_link()
    if not prog:
        pytest.skip("reference sources not present")
    r = subprocess.run([prog], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stdout
    nm = subprocess.run(["nm", "-D", "--undefined-only", prog], capture_output=True, text=True,
                        check=True).stdout
    wanted = {"init_gaugefixing", "finalize_gaugefixing", "overrelax_gauge", "calc_plaquette",
              "simannealing_gauge", "init_MT", "gfx_legacy_get_trafo", "limeCreateReader",
              "limeReaderReadData", "limeCreateWriter", "limeWriteRecordData"}
    undefined = {line.split()[-1].split("@")[0] for line in nm.splitlines() if line.strip()}
    assert wanted <= undefined
    lib = ctypes.CDLL(gfx.library_path())
    system = [ctypes.CDLL(None), ctypes.CDLL("libm.so.6")]
    for s in sorted(undefined):
        if s.startswith("_") or any(hasattr(x, s) for x in system):
            continue  # C runtime and math library
        assert hasattr(lib, s), s
