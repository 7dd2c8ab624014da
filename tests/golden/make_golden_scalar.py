"""Generate the golden vectors that pin the scalar-advection oracle to the reference.

Runs the reference's own scalar-advection code (oracle/_ref/libhcref_scalar.so,
built by oracle/ref/build_ref.sh from the reference headers where they lie) --
the Rusanov and central fluxes and the Riemann (inflow/outflow) ghost update in
the conserved basis {u, v, q} -- on seeded inputs and stores inputs and outputs
in scalar_golden.npz.  Only this script needs the reference tree.

    python tests/golden/make_golden_scalar.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scalar_golden.npz")
SO = os.path.join(ROOT, "oracle", "_ref", "libhcref_scalar.so")


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    lib = C.CDLL(SO)
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    lib.ref_scalar_flux.argtypes = [C.c_int, dp, dp, dp, dp]
    lib.ref_scalar_bc_riemann.argtypes = [dp, dp, dp, dp]
    rng = np.random.default_rng(20261204)
    n = 4000
    th = rng.uniform(-np.pi, np.pi, n)
    faces = np.stack([rng.uniform(0.05, 2.0, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n),
                      np.cos(th), np.sin(th), -np.sin(th), np.cos(th)], axis=1)
    ql = rng.uniform(-1.5, 1.5, (n, 3))
    qr = rng.uniform(-1.5, 1.5, (n, 3))
    qr[: n // 10, :2] = ql[: n // 10, :2]  # uniform advecting velocity across the face
    g = {"faces": faces, "ql": ql, "qr": qr}
    for kind in (0, 1):
        out = np.empty((n, 4))
        for m in range(n):
            lib.ref_scalar_flux(kind, np.ascontiguousarray(faces[m]), ql[m].copy(), qr[m].copy(), out[m])
        g[f"flux_{kind}"] = out
    out = np.empty((n, 3))
    for m in range(n):
        lib.ref_scalar_bc_riemann(np.ascontiguousarray(faces[m]), ql[m].copy(), qr[m].copy(), out[m])
    g["riemann"] = out
    np.savez_compressed(OUT, **g)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
