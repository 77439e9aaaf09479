"""Generates the golden fixtures in tests/golden/ from the CPU oracle.

The reference (Python + NVIDIA Warp) cannot run on these machines and ships no
fixtures of its own, so these vectors are produced by the oracle
(oracle/flub_oracle.c, FP32 and FP64), whose correctness is pinned separately by
tests/test_oracle_kat.py (hand-derived known answers and an independent NumPy
restatement).  Each fixture stores its inputs, so the GPU parity tests do not
depend on regenerating scenes bit for bit on another platform.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from flub_gb300 import scenes  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    "box16_l3": lambda: scenes.box(16, seed=10, levels=3),
    "sphere16_l2": lambda: scenes.sphere(16, seed=11, levels=2),
    "dam32_l3": lambda: scenes.dam(32, seed=12, levels=3),
    "rand16_l3": lambda: scenes.random_scene(16, 13, levels=3),
}


def make(name, s):
    out = O.project(s, max_iters=200, rel_tol=1e-12, abs_tol=0.0)
    out64 = O.project(s, max_iters=200, rel_tol=1e-12, abs_tol=0.0, dtype=np.float64)
    z = O.vcycle(out["r0"], out["tags"], np.float32)
    ap = O.matvec(z, out["tag"])
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"),
        levels=np.int32(s.levels), h=np.float64(s.h), phi=s.phi, prims=s.prims.view(np.uint8),
        u=s.u, v=s.v, w=s.w, ur=s.ur, vr=s.vr, wr=s.wr,
        tag=out["tag"], phi_rigid=out["phi_rigid"], div=out["div"], r0=out["r0"], vcycle_r0=z, matvec_z=ap,
        x=out["x"], x64=out64["x"].astype(np.float64), iters=np.int32(out["iters"]),
        iters64=np.int32(out64["iters"]), u_out=out["u"], v_out=out["v"], w_out=out["w"])
    print(f"{name}: iters {out['iters']} (fp64 {out64['iters']}), fluid {int((out['tag'] == 1).sum())}")


def load(name):
    d = dict(np.load(os.path.join(HERE, f"{name}.npz")))
    d["prims"] = d["prims"].view(scenes.PRIM_DTYPE)
    return d


if __name__ == "__main__":
    for name, fn in CASES.items():
        make(name, fn())
