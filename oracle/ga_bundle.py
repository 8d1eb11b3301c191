"""Named-array bundle files exchanged with the reference harness.

TEST INFRASTRUCTURE.  Format: b"GABN", uint32 record count, then per record
char name[32] (NUL padded), int64 n, float64 data[n] (little endian).
"""
from __future__ import annotations

import struct

import numpy as np


def write_bundle(path, arrays: dict) -> None:
    with open(path, "wb") as fp:
        fp.write(b"GABN")
        fp.write(struct.pack("<I", len(arrays)))
        for name, val in arrays.items():
            a = np.ascontiguousarray(np.asarray(val, dtype="<f8").ravel())
            nb = name.encode()
            if len(nb) > 31:
                raise ValueError(f"name too long: {name}")
            fp.write(nb + b"\0" * (32 - len(nb)))
            fp.write(struct.pack("<q", a.size))
            fp.write(a.tobytes())


def read_bundle(path) -> dict:
    out = {}
    with open(path, "rb") as fp:
        if fp.read(4) != b"GABN":
            raise ValueError(f"{path}: not a bundle")
        (count,) = struct.unpack("<I", fp.read(4))
        for _ in range(count):
            name = fp.read(32).split(b"\0", 1)[0].decode()
            (n,) = struct.unpack("<q", fp.read(8))
            out[name] = np.frombuffer(fp.read(8 * n), dtype="<f8").copy()
    return out
