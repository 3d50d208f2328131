"""CPU tests of the C ABI: the library loads, exports every declared entry
point, and its host-only functions (parser, .bin I/O, size checks) agree with
the oracle.  No kernel runs here."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import cdi_oracle as O

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(cdx_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol(cdx):
    lib = cdx.lib()
    decl = declared_symbols()
    assert decl, "no declarations found"
    for name in decl:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(cdx.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(cdx_\w+)", out))
    assert decl <= exported
    assert set(cdx.exported_symbols()) <= exported


REF_STRINGS = [
    "100*(3*POSHIO+20*RAAR+1*POSHIO+1*shrinkWrap)+20*RAAR+1*ER",
    "200*(20*POSHIO+1*POSHIO+1*shrinkWrap)+100*POSHIO",
    "3000*RAAR+20*ER",
    "5*(20*HIO+1*shrinkWrap)+20*ER",
    "2*(1*HIO+1*ER)+3*(1*RAAR)+1*KKT+1*XCORRELATION+1*FHIO+1*POSER+1*TV",
    "0*HIO+4*ER",
]


@pytest.mark.parametrize("s", REF_STRINGS)
def test_parser_matches_oracle(cdx, s):
    assert cdx.algo_expand(s) == O.AlgoParser(s).expand()


def test_parser_nested_groups_and_errors(cdx):
    s = "5*(9*(20*HIO+1*shrinkWrap)+20*ER+1*shrinkWrap)"
    inner = [O.HIO] * 20 + [O.SHRINKWRAP]
    assert cdx.algo_expand(s) == (inner * 9 + [O.ER] * 20 + [O.SHRINKWRAP]) * 5
    for bad in ["10*BOGUS", "HIO", "3*HIO+", "2*(1*HIO", "1*HIO+0*ER", "-1*HIO", ""]:
        with pytest.raises(cdx.CdxError) as e:
            cdx.algo_expand(bad)
        assert e.value.code in (cdx.CDX_ERR_ALGO, cdx.CDX_ERR_ARG)


def test_bin_io_interoperates_with_oracle(cdx, tmp_path):
    a = (np.random.default_rng(0).standard_normal((6, 10)) + 1j).astype(np.complex64)
    cdx.write_bin(tmp_path / "a.bin", a)
    assert np.array_equal(O.read_bin(tmp_path / "a.bin"), a)
    r = np.random.default_rng(1).random((5, 7)).astype(np.float32)
    O.write_bin(tmp_path / "r.bin", r)
    assert np.array_equal(cdx.read_bin(tmp_path / "r.bin"), r)
    (tmp_path / "bad.bin").write_bytes(b"\x07" + b"\0" * 19)
    with pytest.raises(cdx.CdxError) as e:
        cdx.read_bin(tmp_path / "bad.bin")
    assert e.value.code == cdx.CDX_ERR_IO
    with pytest.raises(cdx.CdxError):
        cdx.read_bin(tmp_path / "missing.bin")
    short = tmp_path / "short.bin"
    short.write_bytes((tmp_path / "a.bin").read_bytes()[:40])
    with pytest.raises(cdx.CdxError):
        cdx.read_bin(short)


def test_size_support(cdx):
    lib = cdx.lib()
    for n in [16, 24, 128, 192, 256, 384, 512, 2048, 3072, 4096]:
        assert lib.cdx_size_supported(n) == 1
    for n in [8, 100, 250, 5000, 8192, 640]:
        assert lib.cdx_size_supported(n) == 0
    # size errors are reported before any device work
    p = cdx.Params()
    lib.cdx_params_default(ctypes.byref(p))
    p.rows, p.cols = 250, 256
    h = ctypes.c_void_p()
    assert lib.cdx_create(ctypes.byref(p), None, ctypes.byref(h)) == cdx.CDX_ERR_SIZE
    assert b"250" in lib.cdx_last_error()


def test_default_params(cdx):
    p = cdx.default_params(256, 256)
    assert p.beta == 1.0 and p.rcolor == 65535 and p.sigma0 == 3.0 and p.sigma_min == 2.0
    assert abs(p.sigma_decay - 0.99) < 1e-7 and p.batch == 1 and p.use_graph == 1


def test_tuning_file_round_trip(cdx, tmp_path):
    """The autotuner's JSON file: a file in the documented shape loads, and
    saving writes its entries back; malformed or out-of-range entries are
    refused.  Host-only (no kernel runs)."""
    good = tmp_path / "tune.json"
    good.write_text('{"cdx_tuning": 1, "entries": [\n'
                    '  {"device": "Some GPU", "rows": 256, "cols": 256, "batch": 64, "pdl_col": 1, "pdl_row": 0,'
                    ' "row_chunk_bits": 3, "us": 45.5},\n'
                    '  {"device": "Some GPU", "rows": 192, "cols": 384, "batch": 2, "pdl_col": 0, "pdl_row": 1,'
                    ' "row_chunk_bits": 2, "us": 30.25}]}\n')
    assert cdx.tuning_load(good) == 2
    out = tmp_path / "saved.json"
    cdx.tuning_save(out)
    text = out.read_text()
    for frag in ['"device": "Some GPU", "rows": 256, "cols": 256, "batch": 64, "pdl_col": 1, "pdl_row": 0, '
                 '"row_chunk_bits": 3', '"rows": 192, "cols": 384, "batch": 2, "pdl_col": 0, "pdl_row": 1, '
                 '"row_chunk_bits": 2']:
        assert frag in text
    assert cdx.tuning_load(out) == 2
    bad = tmp_path / "bad.json"
    for body in ['{"entries": [{"device": "X", "rows": 256, "cols": 256, "batch": 1, "pdl_col": 0, "pdl_row": 0,'
                 ' "row_chunk_bits": 9}]}',                     # 9 > the chunk bits 256 allows
                 '{"entries": [{"device": "X", "rows": 250, "cols": 256, "batch": 1, "pdl_col": 0, "pdl_row": 0,'
                 ' "row_chunk_bits": 1}]}',                     # unsupported length
                 '{"entries": [ {"device": "X", "rows": 256 ', '[]']:
        bad.write_text(body)
        with pytest.raises(cdx.CdxError):
            cdx.tuning_load(bad)
