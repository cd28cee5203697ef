"""Reader/writer for the tagged binary dumps the oracle's reference driver
writes (oracle/ref_driver.cpp), and writer for its input files.

Record layout: 32-byte name, int32 type code (1 int32, 2 int64, 3 float64),
int64 count, payload.
"""
import struct

import numpy as np

_DT = {1: np.int32, 2: np.int64, 3: np.float64}


def read_dump(path):
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    off = 0
    while off < len(buf):
        name = buf[off:off + 32].split(b"\0", 1)[0].decode()
        code, count = struct.unpack_from("<iq", buf, off + 32)
        off += 44
        dt = np.dtype(_DT[code])
        n = count * dt.itemsize
        out[name] = np.frombuffer(buf, dtype=dt, count=count, offset=off).copy()
        off += n
    return out


def csr(d, name):
    """Return the per-(level, box) lists of a CSR record pair as a list."""
    ptr, val = d[name + ".ptr"], d[name + ".val"]
    return [val[ptr[i]:ptr[i + 1]] for i in range(len(ptr) - 1)]


def _f64(v):
    """Real vectors as doubles; complex ones as interleaved (re, im) doubles."""
    if np.iscomplexobj(v):
        return np.ascontiguousarray(v, dtype=np.complex128).view(np.float64)
    return np.ascontiguousarray(v, dtype=np.float64)


def write_input(path, points=None, vecs=(), xtrue=None, dense=False):
    with open(path, "wb") as f:
        if points is None:
            f.write(struct.pack("<q", 0))
        else:
            p = np.ascontiguousarray(points, dtype=np.float64)
            f.write(struct.pack("<q", p.shape[0]))
            f.write(p.tobytes())
        vecs = [_f64(v) for v in vecs]
        f.write(struct.pack("<q", len(vecs)))
        for v in vecs:
            f.write(v.tobytes())
        if xtrue is None:
            f.write(struct.pack("<q", 0))
        else:
            f.write(struct.pack("<q", 1))
            f.write(_f64(xtrue).tobytes())
        f.write(struct.pack("<q", 1 if dense else 0))
