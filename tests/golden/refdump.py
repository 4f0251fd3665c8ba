"""Reader for the binary records written by oracle/ref_driver.cpp."""
from __future__ import annotations

import numpy as np


def read_dump(path: str) -> dict:
    with open(path, "rb") as f:
        buf = f.read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(buf, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a.copy()

    n, nnb, nnz = take(np.int64, 3)
    time, courant = take(np.float64, 2)
    (dlc,) = take(np.int64, 1)
    d = dict(time=float(time), courant=float(courant), debug_log_count=int(dlc))
    d["pos"] = take(np.float64, 3 * n).reshape(n, 3)
    d["vel"] = take(np.float64, 3 * n).reshape(n, 3)
    d["pressure"] = take(np.float64, n)
    d["min_pressure"] = take(np.float64, n)
    d["ndr"] = take(np.float64, n)
    d["type"] = take(np.int32, n)
    d["bc"] = take(np.int32, n)
    d["dirichlet"] = take(np.int32, n)
    d["nb_off"] = take(np.int64, n + 1)
    d["nb_id"] = take(np.int32, nnb)
    d["nb_dist"] = take(np.float64, nnb)
    d["source"] = take(np.float64, n)
    d["row_ptr"] = take(np.int64, n + 1)
    d["col"] = take(np.int32, nnz)
    d["val"] = take(np.float64, nnz)
    assert off == len(buf), (off, len(buf))
    return d
