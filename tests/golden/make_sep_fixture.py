"""Writes the SEP dataset fixture sep_tiny.H / sep_tiny.H@ by hand, with no
use of the library: a header in the published SEP form (appended history:
n2 is set twice and the later value counts; quoted and unquoted values; a
word without '='; a relative in=) and 4 x 3 x 2 big-endian xdr_float values
v = 100 i3 + 10 i2 + i1 + 0.25.  Run from this directory:
python make_sep_fixture.py"""
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

HEADER = """sep_tiny history
n1=4 o1=0.0 d1=0.004 label1="time (s)"
n2=7
Appended by a later program:
n2=3 o2=-25.0 d2=12.5 label2='offset'
n3=2 o3=100 d3=25 label3=y esize=4
data_format="xdr_float" in=sep_tiny.H@
"""


def values():
    i3, i2, i1 = np.meshgrid(np.arange(2), np.arange(3), np.arange(4), indexing="ij")
    return (100 * i3 + 10 * i2 + i1 + 0.25).astype(np.float32)


if __name__ == "__main__":
    (HERE / "sep_tiny.H").write_text(HEADER)
    values().astype(">f4").tofile(HERE / "sep_tiny.H@")
