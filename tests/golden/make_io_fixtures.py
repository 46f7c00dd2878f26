"""Generate tests/golden/io_reference.json: what the reference's own file code
(gauge_io.c, spinor_io.c, cksum.c, compiled unchanged into oracle/_ref/libref_io.so
with libgfx's LIME records in place of c-lime) writes and reads.

Run here, where the reference sources are present:
    python tests/golden/make_io_fixtures.py
The lattice is 4x2x2x4 with exactly representable values (so the 32-bit file is
exact too); the hashes are sha256 of the files the reference writes.
"""
import ctypes
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

DIMS = (4, 2, 2, 4)
PLAQ, BETA = 0.5872, 6.0


def field(dims, per_site=4):
    """per_site su3 per site with values k/256 for small integers k"""
    n = per_site * int(np.prod(dims)) * 18
    k = np.arange(n, dtype=np.int64)
    return (((k * 7919) % 2001) - 1000).astype(np.float64) / 256.0


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main():
    from oracle import build as ob
    lib_path = ob.build_reference_io()
    if not lib_path:
        raise SystemExit("reference sources not present")
    ref = ctypes.CDLL(lib_path, mode=ctypes.RTLD_LOCAL)
    dp = ctypes.POINTER(ctypes.c_double)
    d4 = (ctypes.c_int * 4)(*DIMS)
    u = field(DIMS)
    out = {"dims": DIMS, "plaquette": PLAQ, "beta": BETA, "files": {}, "cksum": {}}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            for prec in (64, 32):
                name = "conf_%d.ildg" % prec
                a = u.copy()
                assert ref.ref_io_write_ildg(name.encode(), d4, a.ctypes.data_as(dp), prec,
                                             ctypes.c_double(PLAQ), ctypes.c_double(BETA)) == 0
                out["files"][name] = sha(name)
            # the reference reader on its own 64-bit file
            back = np.zeros_like(u)
            pl, be = ctypes.c_double(), ctypes.c_double()
            assert ref.ref_io_read_ildg(b"conf_64.ildg", d4, back.ctypes.data_as(dp),
                                        ctypes.byref(pl), ctypes.byref(be)) == 0
            out["ildg64_read_back_equal"] = bool(np.array_equal(back, u))
            out["ildg64_read_plaquette"] = pl.value
            out["ildg64_read_beta"] = be.value
            a = u.copy()
            assert ref.ref_io_write_bqcd(b"conf", d4, a.ctypes.data_as(dp), ctypes.c_double(PLAQ),
                                         ctypes.c_double(BETA)) == 0
            assert np.array_equal(a, u)  # restored after the in-place byte swap
            for t in range(DIMS[3]):
                name = "conf.%03d.u" % t
                out["files"][name] = sha(name)
            out["files"]["conf.info"] = sha("conf.info")
            out["info_text"] = open("conf.info").read()
            sums = (ctypes.c_ulong * DIMS[3])()
            back = np.zeros_like(u)
            assert ref.ref_io_read_bqcd(b"conf", d4, back.ctypes.data_as(dp), sums) == 0
            out["bqcd_read_back_equal"] = bool(np.array_equal(back, u))
            out["bqcd_read_sums"] = list(sums)
        finally:
            os.chdir(cwd)
    for label, data in [("empty", b""), ("hello", b"hello world\n"),
                        ("bytes0-255", bytes(range(256))), ("field", u.tobytes())]:
        crc, nb = ctypes.c_ulong(), ctypes.c_ulong()
        buf = ctypes.create_string_buffer(data, len(data))
        ref.ref_io_cksum(buf, ctypes.c_long(len(data)), ctypes.byref(crc), ctypes.byref(nb))
        out["cksum"][label] = [crc.value, nb.value]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io_reference.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", path)


if __name__ == "__main__":
    main()
