"""Bit-pattern equality of floating-point arrays: unlike np.array_equal it
tells +0 from -0 (and compares NaNs by payload), which is what bit-exact
parity with the oracle means."""
import numpy as np

_UINT = {2: np.uint16, 4: np.uint32, 8: np.uint64}


def same_bits(got, want) -> bool:
    g = np.ascontiguousarray(got)
    w = np.ascontiguousarray(want, dtype=g.dtype)
    if g.shape != w.shape:
        return False
    if g.dtype.kind != "f":
        return bool(np.array_equal(g, w))
    u = _UINT[g.dtype.itemsize]
    return bool(np.array_equal(g.view(u), w.view(u)))
