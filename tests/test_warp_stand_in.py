"""The CPU stand-in for ``warp`` (oracle/warp_cpu, test infrastructure for the
reference-made golden fixtures): kernel and func bodies evaluate float
literals and module-level Python floats as FP32 constants, as Warp's code
generator does, while the module's host code keeps Python's doubles; FP32
scalars combine with vectors as vectors.  Run in a child process so that the
stand-in's ``warp`` never enters this one."""
import multiprocessing as mp
import os
import sys
import textwrap

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STAND_IN = os.path.join(os.path.dirname(HERE), "oracle", "warp_cpu")

MODULE = textwrap.dedent('''
    import warp as wp

    C = 0.1  # a module-level Python float

    @wp.func
    def third(x: float):
        return x * (1.0 / 3.0)

    @wp.kernel
    def k(out: wp.array(dtype=float), vout: wp.array(dtype=wp.vec3)):
        i = wp.tid()
        out[0] = 0.1 / 0.3
        out[1] = C * 9.0
        out[2] = float(i) + 0.1
        out[3] = third(1.0)
        vout[0] = (0.5 * C) * wp.vec3(1.0, 2.0, 3.0)

    def host():
        return C * 9.0
''')


def _child(moddir, q):
    sys.dont_write_bytecode = True
    sys.path.insert(0, moddir)
    sys.path.insert(0, STAND_IN)
    import warp as wp
    import stand_in_probe as m
    out = wp.zeros(4, dtype=float)
    vout = wp.zeros(1, dtype=wp.vec3)
    wp.launch(m.k, dim=1, inputs=[out, vout])
    v = vout[0]
    q.put((out.numpy().copy(), type(v).__name__, [float(c) for c in v], type(m.host()).__name__, m.host()))


def test_kernel_constants_are_fp32_and_host_code_is_not(tmp_path):
    (tmp_path / "stand_in_probe.py").write_text(MODULE)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_child, args=(str(tmp_path), q))
    p.start()
    out, vtype, vec, host_type, host_val = q.get(timeout=120)
    p.join()
    f = np.float32
    # FP32 operations, not a double folded by Python and rounded once: the
    # two differ for these operands
    assert out[0] == f(0.1) / f(0.3) and out[0] != f(0.1 / 0.3)
    assert out[1] == f(0.1) * f(9.0) and out[1] != f(0.1 * 9.0)
    assert out[2] == f(0.0) + f(0.1)
    assert out[3] == f(1.0) * (f(1.0) / f(3.0))
    assert vtype == "vec3"
    s = f(0.5) * f(0.1)
    assert vec == [float(s * f(1.0)), float(s * f(2.0)), float(s * f(3.0))]
    assert host_type == "float" and host_val == 0.1 * 9.0  # a double, as Python computes it
