"""NPY header rules of numrs2's io::npy_npz restated in Python (test
infrastructure: the tests compare the library's NPY writer and reader with
these).

construct_npy_header: src/io/npy_npz.rs:48-99.
parse_npy_header:     src/io/npy_npz.rs:263-339.
"""
from __future__ import annotations

import struct

MAGIC = b"\x93NUMPY"


def construct_npy_header(descr: str, shape) -> bytes:
    """{'descr': ..., 'fortran_order': False, 'shape': (...), } padded with
    16 - ((len + 10) % 16) spaces (16 when already aligned), version 1.0,
    little-endian u16 length, no trailing newline."""
    d = "{'descr': '%s', 'fortran_order': False, 'shape': (" % descr
    for i, dim in enumerate(shape):
        if i > 0:
            d += ", "
        d += str(int(dim))
        if len(shape) == 1:
            d += ","
    d += "), }"
    d += " " * (16 - ((len(d) + 10) % 16))
    return MAGIC + bytes([1, 0]) + struct.pack("<H", len(d)) + d.encode()


def parse_npy_header(header: bytes):
    """(shape, descr) by the reference's string search; raises ValueError
    where the reference returns a DeserializationError."""
    if len(header) < 8 or header[:6] != MAGIC:
        raise ValueError("Invalid NPY file: missing magic string")
    if header[6] != 1 or header[7] != 0:
        raise ValueError(f"Unsupported NPY version: {header[6]}.{header[7]}")
    hl = struct.unpack("<H", header[8:10])[0]
    if len(header) < 10 + hl:
        raise ValueError("Invalid NPY file: header too short")
    d = header[10:10 + hl].decode()
    i = d.index("'descr': '") + len("'descr': '")
    descr = d[i:d.index("'", i)]
    j = d.index("'shape': (") + len("'shape': (")
    shape_str = d[j:d.index(")", j)].strip()
    shape = [int(t.strip()) for t in shape_str.split(",") if t.strip()]
    return shape, descr
