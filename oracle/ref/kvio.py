"""Named-array container ("DRKV") read/written by oracle/ref/ref_driver.cpp.

Test infrastructure only (fixture generation).  Layout matches kvio.h.
"""
import struct

import numpy as np

_DT = {0: np.float32, 1: np.int32, 2: np.uint32, 3: np.float64}
_CODE = {np.dtype(np.float32): 0, np.dtype(np.int32): 1, np.dtype(np.uint32): 2, np.dtype(np.float64): 3}


def save(path, items):
    with open(path, "wb") as f:
        f.write(b"DRKV")
        f.write(struct.pack("<I", len(items)))
        for name, arr in items.items():
            arr = np.ascontiguousarray(arr)
            if arr.dtype not in _CODE:
                raise TypeError(f"{name}: unsupported dtype {arr.dtype}")
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)))
            f.write(nb)
            f.write(struct.pack("<IQ", _CODE[arr.dtype], arr.size))
            f.write(arr.tobytes())


def load(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    if data[:4] != b"DRKV":
        raise ValueError("bad magic")
    (n,) = struct.unpack_from("<I", data, 4)
    off = 8
    for _ in range(n):
        (ln,) = struct.unpack_from("<I", data, off)
        off += 4
        name = data[off:off + ln].decode()
        off += ln
        dt, cnt = struct.unpack_from("<IQ", data, off)
        off += 12
        dtype = np.dtype(_DT[dt])
        nbytes = cnt * dtype.itemsize
        out[name] = np.frombuffer(data[off:off + nbytes], dtype=dtype).copy()
        off += nbytes
    return out
