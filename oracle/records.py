"""Record files exchanged with the reference harness (test infrastructure).

Format: b"CFXREC1\\n", then records of
    char name[32]; char dtype[8] ("i4" | "f8" | "s"); int64 count; data.
"""
import struct

import numpy as np

MAGIC = b"CFXREC1\n"


def write(path, recs):
    with open(path, "wb") as fh:
        fh.write(MAGIC)
        for name, val in recs.items():
            if isinstance(val, str):
                data = val.encode()
                dt, n = b"s", len(data)
            else:
                arr = np.ascontiguousarray(val)
                if arr.dtype.kind in "iub":
                    arr = arr.astype(np.int32)
                    dt = b"i4"
                else:
                    arr = arr.astype(np.float64)
                    dt = b"f8"
                data = arr.tobytes()
                n = arr.size
            fh.write(name.encode().ljust(32, b"\0"))
            fh.write(dt.ljust(8, b"\0"))
            fh.write(struct.pack("<q", n))
            fh.write(data)


def read(path):
    out = {}
    with open(path, "rb") as fh:
        if fh.read(8) != MAGIC:
            raise ValueError("bad record file " + path)
        while True:
            hdr = fh.read(48)
            if len(hdr) < 48:
                break
            name = hdr[:32].rstrip(b"\0").decode()
            dt = hdr[32:40].rstrip(b"\0").decode()
            (n,) = struct.unpack("<q", hdr[40:48])
            if dt == "f8":
                out[name] = np.frombuffer(fh.read(8 * n), dtype=np.float64).copy()
            elif dt == "i4":
                out[name] = np.frombuffer(fh.read(4 * n), dtype=np.int32).copy()
            else:
                out[name] = fh.read(n).decode()
    return out
