"""Host-side compatibility pieces: the reference's `input` file format and
the gfortran record framing used by the restart files."""
import struct

import numpy as np

from fortran_records import read_records
from tristan_gb300.config import from_input, parse_input

INPUT = """
#
<time>
c	= .45			# velocity of light
<grid>
mx0 	= 128 		# cells in x
my0 	= 96
mz0 	= 1 			# ignored in 2D
<algorithm>
Corr		= 1.025
ntimes		= 32		# filter passes
<boundaries>
periodicx	= 0
periodicy	= 1
<particles>
ppc0 	= 16
delgam 	= 2.e-5	         # kT/mc^2
gamma0	= 0.5
c_omp	= 10
"""


def test_input_file_parsing(tmp_path):
    p = tmp_path / "input"
    p.write_text(INPUT)
    d = parse_input(str(p))
    assert d["grid"]["mx0"] == 128 and d["algorithm"]["Corr"] == 1.025 and d["particles"]["delgam"] == 2e-5
    cfg = from_input(str(p), dims=2, order=3)
    assert (cfg.nx, cfg.ny, cfg.ntimes, cfg.periodic[:2]) == (128, 96, 32, (0, 1))
    assert (cfg.mx, cfg.my, cfg.mz) == (135, 103, 1)
    assert cfg.gamma_drift > 1.15  # gamma0 < 1 read as v/c


def frame(payload: bytes, max_sub: int) -> bytes:
    """gfortran framing of one record, written independently of the reader"""
    chunks = [payload[i:i + max_sub] for i in range(0, len(payload), max_sub)] or [b""]
    out = b""
    for i, ch in enumerate(chunks):
        lead = len(ch) if i == len(chunks) - 1 else -len(ch)
        tail = len(ch) if i == 0 else -len(ch)
        out += struct.pack("<i", lead) + ch + struct.pack("<i", tail)
    return out


def test_record_reader_with_subrecords(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.bytes(1000)
    b = rng.bytes(10)
    p = tmp_path / "f.d"
    p.write_bytes(frame(a, 300) + frame(b, 4096) + frame(b"", 16))
    recs = read_records(str(p))
    assert recs == [a, b, b""]
