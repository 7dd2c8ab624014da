"""Generate the golden vectors that pin the CPU oracle to the reference.

Runs the reference's own pointwise code (oracle/_ref/libhcref.so, built by
oracle/ref/build_ref.sh from the reference headers where they lie) on seeded
random inputs and stores inputs and outputs in pointwise_golden.npz.  Only this
script needs the reference tree; the tests read the committed .npz.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle_py  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pointwise_golden.npz")
REF_FLUXES = [0, 2, 3, 4, 5, 6]       # Roe, SLAU (literal), AUSM+up, Rusanov, Central, RoeUnprecWS
REF_LIMITERS = [0, 1, 2, 3, 4, 5, 6, 8, 9]


def random_prims(rng, n, gamma=1.4):
    """Primitive states {u, v, rho, p} spanning sub- and supersonic flow."""
    rho = rng.uniform(0.2, 3.0, n)
    p = rng.uniform(0.1, 3.0, n)
    a = np.sqrt(gamma * p / rho)
    mach = rng.uniform(0.0, 2.5, n)
    th = rng.uniform(0, 2 * np.pi, n)
    u = mach * a * np.cos(th)
    v = mach * a * np.sin(th)
    q = np.stack([u, v, rho, p], axis=1)
    q[: n // 20, 0:2] = 0.0            # a few states at rest
    return q


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    ref = oracle_py.reference_pointwise()
    if ref is None:
        raise SystemExit("reference probe unavailable")
    rng = np.random.default_rng(20261203)
    g = {}
    species = np.array([1.4, 287.058, 0.3])
    g["species"] = species

    # faces from random node pairs, through the reference's geom::surface
    nf = 400
    p0 = rng.uniform(-3, 3, (nf, 2))
    p1 = p0 + rng.uniform(-1, 1, (nf, 2))
    faces = np.stack([ref.surface(p0[k], p1[k]) for k in range(nf)])
    g["surface_p0"], g["surface_p1"], g["surface_out"] = p0, p1, faces

    quads = rng.uniform(-0.2, 0.2, (200, 8)) + np.array([0, 0, 1, 0, 0, 1, 1, 1.0])
    g["volume_in"] = quads
    g["volume_out"] = np.stack([ref.volume(q) for q in quads])

    ql = random_prims(rng, nf)
    qr = random_prims(rng, nf)
    # near-equal pairs exercise the entropy fix and the small-jump branches
    qr[nf // 4: nf // 2] = ql[nf // 4: nf // 2] * (1 + 1e-3 * rng.standard_normal((nf // 4, 4)))
    g["flux_ql"], g["flux_qr"] = ql, qr
    for k in REF_FLUXES:
        g[f"flux_{k}"] = np.stack([ref.flux(k, species, faces[m], ql[m], qr[m]) for m in range(nf)])
    g["exact_flux"] = np.stack([ref.exact_flux(species, faces[m][3:5].copy(), ql[m]) for m in range(nf)])

    ab = rng.standard_normal((600, 2))
    ab[:50, 1] = ab[:50, 0]                     # equal slopes
    ab[50:100, 1] = -ab[50:100, 0]              # opposite slopes
    ab[100:120] = 0.0                            # both zero
    ab[120:140, 0] = 0.0                         # one zero
    ab[140:200, 1] *= 3.0                        # large ratios
    g["limit_ab"] = ab
    for k in REF_LIMITERS:
        g[f"limit_{k}"] = np.array([ref.limit(k, a, b) for a, b in ab])

    g["state_out"] = np.stack([ref.prim2state(species, q) for q in ql])
    g["prim2cons_out"] = np.stack([ref.prim2cons(species, q) for q in ql])
    g["cons2prim_in"] = g["prim2cons_out"] * (1 + 1e-2 * rng.standard_normal((nf, 4)))
    g["cons2prim_out"] = np.stack([ref.cons2prim(species, c) for c in g["cons2prim_in"]])

    din = rng.standard_normal((nf, 4))
    g["delta_in"] = din
    for k in range(4):
        g[f"delta_{k}"] = np.stack([ref.delta(k, species, ql[m], din[m]) for m in range(nf)])

    # boundary updates: far-field states around the interior state, all flow regimes
    qf = random_prims(rng, nf)
    g["bc_qf"] = qf
    for k in (2, 3):
        g[f"bc_{k}"] = np.stack([ref.bc_update(k, species, faces[m], ql[m], qf[m]) for m in range(nf)])
    dq = 0.05 * rng.standard_normal((nf, 4))
    g["wall_dq"] = dq
    g["wall_out"] = np.stack([ref.wall_flux(species, faces[m], ql[m], dq[m]) for m in range(nf)])

    for k in range(4):
        g[f"rk_{k}"] = ref.rk_table(k)
    # RoeUnprecWS at lower cut-off Mach numbers; AUSM+up at its nine (velocity, pressure)
    # low-Mach scalings for three (lref, species dt) pairs
    g["roews_minf"] = np.array([0.05, 1e-3])
    g["roews_out"] = np.stack([np.stack([ref.flux(6, np.array([1.4, 287.058, mi]), faces[m], ql[m], qr[m])
                                         for m in range(nf)]) for mi in g["roews_minf"]])
    ns = 160
    g["ausm_species"] = np.array([[1.4, 287.058, 0.05, 1.0, np.finfo(np.float64).max],
                                  [1.4, 287.058, 0.05, 1.0, 0.5],
                                  [1.4, 287.058, 0.01, 3.0, 0.01]])
    g["ausm_scaled"] = np.stack([np.stack([np.stack([np.stack([
        ref.ausmpup_scaled(vs, ps, sp5, faces[m], ql[m], qr[m]) for m in range(ns)])
        for ps in range(3)]) for vs in range(3)]) for sp5 in g["ausm_species"]])
    # the reference computes SLAU's scalings and never reads them: its nine
    # instantiations are one flux (checked against flux_2 by the tests)
    ref.lib.ref_slau_scaled.argtypes = ref.fn("ausmpup_scaled").argtypes

    def slau_scaled(vs, ps, sp5, m):
        out = np.empty(5)
        ref.lib.ref_slau_scaled(vs, ps, np.asarray(sp5, dtype=np.float64), faces[m], ql[m], qr[m], out)
        return out
    g["slau_scaled"] = np.stack([np.stack([np.stack([np.stack([slau_scaled(vs, ps, sp5, m) for m in range(ns)])
                                                     for ps in range(3)]) for vs in range(3)])
                                 for sp5 in g["ausm_species"]])
    # a solution field in the conserved basis {rho u, rho v, rho, rho E}: fluxes, far-field
    # updates and the wall flux on ConsSets (the reference's functions are generic over
    # the basis and reach the State through set2State)
    cl = np.stack([ref.prim2cons(species, q) for q in ql])
    cr = np.stack([ref.prim2cons(species, q) for q in qr])
    cf = np.stack([ref.prim2cons(species, q) for q in qf])
    g["cons_ql"], g["cons_qr"], g["cons_qf"] = cl, cr, cf
    for k in REF_FLUXES:
        g[f"cons_flux_{k}"] = np.stack([ref.flux_cons(k, species, faces[m], cl[m], cr[m]) for m in range(nf)])
    for k in (2, 3):
        g[f"cons_bc_{k}"] = np.stack([ref.bc_update_cons(k, species, faces[m], cl[m], cf[m]) for m in range(nf)])
    g["cons_wall_out"] = np.stack([ref.wall_flux_cons(species, faces[m], cl[m], dq[m]) for m in range(nf)])
    # one-dimensional fluxes and boundary updates (nDim = 1: {u, rho, p}, the face of a node)
    import ctypes as C
    dpp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ref.lib.ref_flux_1d.argtypes = [C.c_int, dpp, dpp, dpp, dpp]
    ref.lib.ref_bc_update_1d.argtypes = [C.c_int, dpp, C.c_int, dpp, dpp, dpp]
    l1 = np.ascontiguousarray(ql[:, [0, 2, 3]])
    r1 = np.ascontiguousarray(qr[:, [0, 2, 3]])
    g["q1d_l"], g["q1d_r"] = l1, r1

    def call(fn, shape, *args):
        out = np.empty(shape)
        fn(*args, out)
        return out
    for k in REF_FLUXES:
        g[f"flux_1d_{k}"] = np.stack([call(ref.lib.ref_flux_1d, 4, k, species, l1[m], r1[m]) for m in range(nf)])
    for side in (0, 1):
        for k in (2, 3):
            g[f"bc_1d_{side}_{k}"] = np.stack([call(ref.lib.ref_bc_update_1d, 3, k, species, side, l1[m], r1[m])
                                               for m in range(nf)])
    g["cyl_nodes"] = ref.cylinder_nodes(12, 16, 0.5, 20.0)
    g["lin_nodes"] = ref.linspace_nodes(9, 7, 0.0, 10.0, -1.0, 3.0)
    np.savez_compressed(OUT, **g)
    print("wrote", OUT, "with", len(g), "arrays")


if __name__ == "__main__":
    main()
