"""Reader/writer for the named-array container ("NQA1") shared by the golden
fixtures and the oracle tools (the C++ side is oracle/nqa_io.h)."""
import struct

import numpy as np

_CODES = {0: np.int32, 1: np.float64, 2: np.int64, 3: np.float32, 4: np.uint8}
_INV = {np.dtype(v): k for k, v in _CODES.items()}


def load(path):
    out = {}
    with open(path, "rb") as f:
        if f.read(4) != b"NQA1":
            raise ValueError(f"bad magic in {path}")
        while True:
            hdr = f.read(4)
            if len(hdr) < 4:
                break
            (nl,) = struct.unpack("<I", hdr)
            name = f.read(nl).decode()
            (dt,) = struct.unpack("<B", f.read(1))
            (cnt,) = struct.unpack("<Q", f.read(8))
            dtype = np.dtype(_CODES[dt])
            out[name] = np.frombuffer(f.read(cnt * dtype.itemsize), dtype=dtype).copy()
    return out


def save(path, arrays):
    with open(path, "wb") as f:
        f.write(b"NQA1")
        for name, arr in arrays.items():
            a = np.ascontiguousarray(arr)
            if a.dtype == np.bool_:
                a = a.astype(np.uint8)
            if a.dtype not in _INV:
                if np.issubdtype(a.dtype, np.integer):
                    a = a.astype(np.int64)
                else:
                    a = a.astype(np.float64)
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)))
            f.write(nb)
            f.write(struct.pack("<B", _INV[a.dtype]))
            f.write(struct.pack("<Q", a.size))
            f.write(a.reshape(-1).tobytes())
