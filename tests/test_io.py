"""Gauge-field files.  CPU tests: the LIME record framing against the record format,
the POSIX cksum against known answers and the reference's cksum.c, and libgfx's
ILDG and BQCD writers byte for byte against the files the reference's own
gauge_io.c writes (hashes in tests/golden/io_reference.json, made by
tests/golden/make_io_fixtures.py), readers and error paths.  GPU tests: loading
links into a context, the gauge-fixed field written from the device, and a
checkpoint that continues bit for bit."""
import hashlib
import json
import os
import struct
import subprocess

import numpy as np
import pytest

import cudagfx_gb300 as gfx

HERE = os.path.dirname(os.path.abspath(__file__))
REF = json.load(open(os.path.join(HERE, "golden", "io_reference.json")))
DIMS = tuple(REF["dims"])
PLAQ, BETA = REF["plaquette"], REF["beta"]


def field(dims, per_site=4):
    """the fixture's field: values k/256 for small integers k (exact in float)"""
    n = per_site * int(np.prod(dims)) * 18
    k = np.arange(n, dtype=np.int64)
    return ((((k * 7919) % 2001) - 1000).astype(np.float64) / 256.0).reshape(-1, 3, 3, 2)


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------
def test_cksum_known_answers_and_reference():
    assert gfx.cksum(b"") == (4294967295, 0)
    assert gfx.cksum(b"hello world\n") == (3733384285, 12)
    data = {"empty": b"", "hello": b"hello world\n", "bytes0-255": bytes(range(256)),
            "field": field(DIMS).tobytes()}
    for label, (crc, nb) in REF["cksum"].items():
        assert gfx.cksum(data[label]) == (crc, nb), label


def test_cksum_matches_cksum_utility(tmp_path):
    p = tmp_path / "x.bin"
    blob = bytes((i * 37 + 11) % 256 for i in range(100003))
    p.write_bytes(blob)
    try:
        out = subprocess.run(["cksum", str(p)], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("no cksum utility")
    crc, n = out.split()[:2]
    assert gfx.cksum(blob) == (int(crc), int(n))


def test_lime_record_framing(tmp_path):
    """header = magic, version 1, MB/ME flags, big-endian length, 128-byte type;
    data zero-padded to 8 bytes (the LIME record format)"""
    p = tmp_path / "f.ildg"
    gfx.ildg_write(str(p), DIMS, field(DIMS), 64, PLAQ, BETA)
    raw = p.read_bytes()
    off, types = 0, []
    while off < len(raw):
        magic, ver, flags, n = struct.unpack(">IHHQ", raw[off:off + 16])
        assert (magic, ver, flags) == (0x456789AB, 1, 0xC000)
        t = raw[off + 16:off + 144].rstrip(b"\0").decode()
        types.append((t, n))
        pad = (8 - n % 8) % 8
        assert raw[off + 144 + n:off + 144 + n + pad] == b"\0" * pad
        off += 144 + n + pad
    assert off == len(raw)
    V = int(np.prod(DIMS))
    assert [t for t, _ in types] == ["ildg-format", "xlf-info", "ildg-binary-data"]
    assert types[2][1] == 4 * V * 144
    # big-endian doubles in ILDG site order (4*pos + mu)
    data = np.frombuffer(raw[-4 * V * 144:], dtype=">f8")
    assert np.array_equal(data, field(DIMS).ravel())


@pytest.mark.parametrize("prec", [64, 32])
def test_ildg_writer_is_byte_identical_to_reference(tmp_path, prec):
    name = "conf_%d.ildg" % prec
    gfx.ildg_write(str(tmp_path / name), DIMS, field(DIMS), prec, PLAQ, BETA)
    assert sha(tmp_path / name) == REF["files"][name]


@pytest.mark.parametrize("prec", [64, 32])
def test_ildg_read_roundtrip_and_metadata(tmp_path, prec):
    p = str(tmp_path / "c.ildg")
    u = field(DIMS)
    gfx.ildg_write(p, DIMS, u, prec, PLAQ, BETA)
    info = gfx.ildg_read_info(p)
    assert info["dims"] == DIMS and info["precision"] == prec
    assert info["plaquette"] == pytest.approx(PLAQ, abs=1e-6)
    assert info["beta"] == pytest.approx(BETA, abs=1e-6)
    back, _ = gfx.ildg_read(p, DIMS)
    assert np.array_equal(back, u)  # the values are exact in float as well


def test_ildg_float_precision_rounds(tmp_path):
    rng = np.random.default_rng(3)
    u = rng.normal(size=(4 * int(np.prod(DIMS)), 3, 3, 2))
    p = str(tmp_path / "f.ildg")
    gfx.ildg_write(p, DIMS, u, 32)
    back, _ = gfx.ildg_read(p, DIMS)
    assert np.array_equal(back, u.astype(np.float32).astype(np.float64))


def test_bqcd_writer_is_byte_identical_to_reference(tmp_path):
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        cks = gfx.bqcd_write("conf", DIMS, field(DIMS), PLAQ, BETA)
    finally:
        os.chdir(cwd)
    for t in range(DIMS[3]):
        name = "conf.%03d.u" % t
        assert sha(tmp_path / name) == REF["files"][name]
    assert (tmp_path / "conf.info").read_text() == REF["info_text"]
    assert [c["sum"] for c in cks] == REF["bqcd_read_sums"]


def test_bqcd_read_and_info(tmp_path):
    base = str(tmp_path / "conf")
    u = field(DIMS)
    gfx.bqcd_write(base, DIMS, u, PLAQ, BETA)
    back, cks = gfx.bqcd_read(base, DIMS)
    assert np.array_equal(back, u)
    info, cks_file = gfx.bqcd_read_info(base + ".info")
    assert info["dims"] == DIMS and info["run"] == 999
    assert info["beta"] == pytest.approx(BETA, abs=1e-3)
    assert info["plaquette"] == pytest.approx(PLAQ, rel=1e-13)
    assert [c["sum"] for c in cks_file] == [c["sum"] for c in cks]
    assert [c["file"] for c in cks_file] == [c["file"] for c in cks]


def test_bqcd_trafo_roundtrip(tmp_path):
    g = field(DIMS, per_site=1)
    base = str(tmp_path / "gt")
    cks = gfx.bqcd_write_trafo(base, DIMS, g)
    back, cks2 = gfx.bqcd_read_trafo(base, DIMS)
    assert np.array_equal(back, g) and cks == cks2
    assert os.path.getsize(base + ".000.g") == int(np.prod(DIMS[:3])) * 144


def test_io_errors(tmp_path):
    p = str(tmp_path / "c.ildg")
    gfx.ildg_write(p, DIMS, field(DIMS), 64)
    with pytest.raises(gfx.GfxError, match="extents"):
        gfx.ildg_read(p, (4, 4, 2, 4))
    with pytest.raises(gfx.GfxError, match="cannot open"):
        gfx.ildg_read(str(tmp_path / "missing.ildg"), DIMS)
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-1000])
    with pytest.raises(gfx.GfxError, match="truncated"):
        gfx.ildg_read(p, DIMS)
    open(p, "wb").write(b"not a lime file" * 20)
    with pytest.raises(gfx.GfxError):
        gfx.ildg_read(p, DIMS)
    with pytest.raises(gfx.GfxError, match="cannot open"):
        gfx.bqcd_read(str(tmp_path / "nothing"), DIMS)


def test_reference_reader_output_recorded():
    # the reference read its own 64-bit file back unchanged (fixture generation)
    assert REF["ildg64_read_back_equal"] and REF["bqcd_read_back_equal"]
    assert REF["ildg64_read_plaquette"] == pytest.approx(PLAQ, abs=1e-6)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_load_links_and_write_links(tmp_path):
    from conftest import smooth_links
    dims = (4, 4, 4, 8)
    u = smooth_links(dims, 0.3, 5)
    p = str(tmp_path / "in.ildg")
    gfx.ildg_write(p, dims, u, 64, 0.9, 6.0)
    c = gfx.Context(dims, precision=gfx.PREC_MIXED)
    info = c.load_links_ildg(p)
    assert info["dims"] == dims
    got = c.get_links().reshape(-1, 18)
    want = np.asarray(u).reshape(-1, 18)
    assert np.max(np.abs(got[:, :12] - want[:, :12])) == 0  # rows 0,1 stored exactly
    c.write_links_ildg(str(tmp_path / "out.ildg"), 64, 6.0)
    back, info2 = gfx.ildg_read(str(tmp_path / "out.ildg"), dims)
    assert np.array_equal(back, c.get_links())
    assert info2["plaquette"] == pytest.approx(c.plaquette(), abs=1e-6)
    with pytest.raises(gfx.GfxError):
        gfx.Context((4, 4, 4, 4)).load_links_ildg(p)


@pytest.mark.gpu
def test_write_fixed_field_matches_host_trafo(tmp_path, oracle):
    from conftest import haar, smooth_links
    dims = (4, 4, 4, 8)
    u = smooth_links(dims, 0.4, 9)
    g = haar(int(np.prod(dims)), 10)
    c = gfx.Context(dims, precision=gfx.PREC_MIXED)
    c.set_links(u)
    c.set_trafo(g)
    u0, g0 = c.get_links(), c.get_trafo()
    c.write_fixed_ildg(str(tmp_path / "fixed.ildg"), 64, 6.0)
    fixed, info = gfx.ildg_read(str(tmp_path / "fixed.ildg"), dims)
    want = oracle.g_trafo18(oracle.lattice(dims), u0.reshape(-1, 18), g0.reshape(-1, 18))
    assert np.max(np.abs(fixed.reshape(-1, 18) - want)) < 1e-13
    assert info["plaquette"] == pytest.approx(c.plaquette(), abs=1e-6)
    # the context is as it was
    assert np.array_equal(c.get_links(), u0) and np.array_equal(c.get_trafo(), g0)


@pytest.mark.gpu
def test_checkpoint_continues_bit_for_bit(tmp_path, mt_params):
    from conftest import smooth_links
    dims = (4, 4, 4, 8)
    V = int(np.prod(dims))
    a = gfx.Context(dims, precision=gfx.PREC_MIXED)
    a.set_links(smooth_links(dims, 0.3, 11))
    a.set_trafo(gfx.random_init_reference(351, V))
    a.mt_load_params(mt_params)
    a.mt_seed(77)
    a.mt_init(2 * V, 8 * V)
    a.or_sweeps(3, omega=1.7, precision=0)  # g current in FP32

    def steps(c):
        c.sa_halfsweep(0, 2.0, precision=1)
        c.mt_update()
        c.sa_halfsweep(1, 2.0, precision=1)
        c.or_sweeps(2, omega=1.7, precision=0)
        c.thermalize(6.0, 1, variant=gfx.HB_KENNEDY_PENDLETON)
        return c.get_trafo(), c.get_links()

    p = str(tmp_path / "ck.lime")
    a.checkpoint_save(p)
    ga, ua = steps(a)
    b = gfx.Context(dims, precision=gfx.PREC_MIXED)
    b.checkpoint_load(p)
    gb, ub = steps(b)
    assert np.array_equal(ga, gb) and np.array_equal(ua, ub)
    with pytest.raises(gfx.GfxError):
        gfx.Context((4, 4, 4, 4)).checkpoint_load(p)
