"""warp.utils stand-in -- TEST INFRASTRUCTURE ONLY (see warp/__init__.py).

``array_inner`` restates Warp's host path for a scalar FP32 array: a
sequential FP32 sum of the element products in index order, written to
``out[0]`` (the reference calls it at multigrid/mgpcg.py:391,401,416,427,451).
Under CUDA Warp reduces in a tree, in an order this stand-in cannot
reproduce; only the CG scalars alpha and beta depend on it."""
import numpy as np

from . import _enqueue


def array_inner(a, b, out=None, count=None, axis=None):
    fa = np.asarray(a, dtype=np.float32).ravel()
    fb = np.asarray(b, dtype=np.float32).ravel()
    n = fa.size if count is None else int(count)

    def run():
        s = np.float32(0.0)
        for i in range(n):
            s = np.float32(s + fa[i] * fb[i])
        if out is not None:
            out[0] = s
        return s

    if out is None:
        return run()
    _enqueue(run)
    return out
