"""Pin the CPU oracle to the reference: every pointwise function of the oracle
must reproduce the golden vectors produced by the reference's own headers
(tests/golden/make_golden.py) bit for bit."""
import os

import numpy as np
import pytest

from oracle import oracle_py

GOLD = os.path.join(os.path.dirname(__file__), "golden", "pointwise_golden.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def o():
    return oracle_py.pointwise()


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(a, b, equal_nan=True), f"max abs diff {np.nanmax(np.abs(a - b))}"


def test_surface_volume(g, o):
    same([o.surface(a, b) for a, b in zip(g["surface_p0"], g["surface_p1"])], g["surface_out"])
    same([o.volume(q) for q in g["volume_in"]], g["volume_out"])


@pytest.mark.parametrize("kind", [0, 2, 3, 4, 5, 6])
def test_fluxes(g, o, kind):
    f, sp = g["surface_out"], g["species"]
    got = [o.flux(kind, sp, f[m], g["flux_ql"][m], g["flux_qr"][m]) for m in range(len(f))]
    same(got, g[f"flux_{kind}"])


def test_roe_ws_low_mach(g, o):
    f = g["surface_out"]
    for mi, want in zip(g["roews_minf"], g["roews_out"]):
        sp = np.array([1.4, 287.058, mi])
        same([o.flux(6, sp, f[m], g["flux_ql"][m], g["flux_qr"][m]) for m in range(len(f))], want)


def test_slau_scalings_are_one_flux(g, o):
    """Slau<V, P> of the reference for all nine scalings equals the oracle's literal SLAU
    (flux kind 2): the reference leaves SLAU's scaling parameters unused."""
    f = g["surface_out"]
    for sp5, got in zip(g["ausm_species"], g["slau_scaled"]):
        ns = got.shape[2]
        sp = np.asarray(sp5[:3])
        want = np.stack([o.flux(2, sp, f[m], g["flux_ql"][m], g["flux_qr"][m]) for m in range(ns)])
        for vs in range(3):
            for ps in range(3):
                same(got[vs, ps], want)


@pytest.mark.parametrize("vs", [0, 1, 2])
@pytest.mark.parametrize("ps", [0, 1, 2])
def test_ausmpup_scalings(g, o, vs, ps):
    f = g["surface_out"]
    for sp5, want in zip(g["ausm_species"], g["ausm_scaled"]):
        ns = want.shape[2]
        same([o.ausmpup_scaled(vs, ps, sp5, f[m], g["flux_ql"][m], g["flux_qr"][m]) for m in range(ns)],
             want[vs, ps])


@pytest.mark.parametrize("kind", [0, 2, 3, 4, 5, 6])
def test_fluxes_conserved_basis(g, o, kind):
    f, sp = g["surface_out"], g["species"]
    got = [o.flux_cons(kind, sp, f[m], g["cons_ql"][m], g["cons_qr"][m]) for m in range(len(f))]
    same(got, g[f"cons_flux_{kind}"])


@pytest.mark.parametrize("kind", [2, 3])
def test_boundary_updates_conserved_basis(g, o, kind):
    f, sp = g["surface_out"], g["species"]
    same([o.bc_update_cons(kind, sp, f[m], g["cons_ql"][m], g["cons_qf"][m]) for m in range(len(f))],
         g[f"cons_bc_{kind}"])


def test_wall_flux_conserved_basis(g, o):
    f, sp = g["surface_out"], g["species"]
    same([o.wall_flux_cons(sp, f[m], g["cons_ql"][m], g["wall_dq"][m]) for m in range(len(f))], g["cons_wall_out"])


def _emb(q):
    return np.array([q[0], 0.0, q[1], q[2]])


@pytest.mark.parametrize("kind", [0, 2, 3, 4, 5, 6])
def test_one_dimensional_fluxes(g, o, kind):
    """The reference's nDim = 1 fluxes equal the oracle's 2D fluxes with the second velocity
    0 on the face (area 1, normal (1, 0)) of a node: the 1D oracle path reuses them."""
    sp, face = g["species"], np.array([1.0, 0.0, 0.0, 1.0, 0.0, 0.0, 1.0])
    got = []
    for ql, qr in zip(g["q1d_l"], g["q1d_r"]):
        f = o.flux(kind, sp, face, _emb(ql), _emb(qr))
        got.append([f[0], f[2], f[3], f[4]])
    same(got, g[f"flux_1d_{kind}"])


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("kind", [2, 3])
def test_one_dimensional_boundary_updates(g, o, side, kind):
    sp = g["species"]
    n = 1.0 if side == 0 else -1.0  # into the domain
    face = np.array([1.0, 0.0, 0.0, n, 0.0, 0.0, n])
    got = []
    for ql, qr in zip(g["q1d_l"], g["q1d_r"]):
        b = o.bc_update(kind, sp, face, _emb(ql), _emb(qr))
        got.append([b[0], b[2], b[3]])
    same(got, g[f"bc_1d_{side}_{kind}"])


def test_exact_flux(g, o):
    f, sp = g["surface_out"], g["species"]
    same([o.exact_flux(sp, f[m][3:5].copy(), g["flux_ql"][m]) for m in range(len(f))], g["exact_flux"])


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5, 6, 8, 9])
def test_limiters(g, o, kind):
    same([o.limit(kind, a, b) for a, b in g["limit_ab"]], g[f"limit_{kind}"])


def test_transforms(g, o):
    sp = g["species"]
    same([o.prim2state(sp, q) for q in g["flux_ql"]], g["state_out"])
    same([o.prim2cons(sp, q) for q in g["flux_ql"]], g["prim2cons_out"])
    same([o.cons2prim(sp, q) for q in g["cons2prim_in"]], g["cons2prim_out"])
    for k in range(4):
        same([o.delta(k, sp, q, d) for q, d in zip(g["flux_ql"], g["delta_in"])], g[f"delta_{k}"])


@pytest.mark.parametrize("kind", [2, 3])
def test_farfield_updates(g, o, kind):
    f, sp = g["surface_out"], g["species"]
    same([o.bc_update(kind, sp, f[m], g["flux_ql"][m], g["bc_qf"][m]) for m in range(len(f))], g[f"bc_{kind}"])


def test_wall_flux(g, o):
    f, sp = g["surface_out"], g["species"]
    same([o.wall_flux(sp, f[m], g["flux_ql"][m], g["wall_dq"][m]) for m in range(len(f))], g["wall_out"])


def test_rk_tables_and_meshes(g, o):
    for k in range(4):
        same(o.rk_table(k), g[f"rk_{k}"])
    same(o.cylinder_nodes(12, 16, 0.5, 20.0), g["cyl_nodes"])
    same(o.linspace_nodes(9, 7, 0.0, 10.0, -1.0, 3.0), g["lin_nodes"])


def test_vanleer_decision(o):
    """The harmonic-mean van Leer slope used for the van Leer configs, and the
    literal reference expression kept beside it."""
    assert o.limit(7, 0.2, 0.5) == pytest.approx(2 * 0.2 * 0.5 / 0.7)
    assert o.limit(7, 0.2, -0.5) == 0.0
    assert o.limit(8, 0.2, 0.5) == pytest.approx((0.5 + 0.5) / (0.2 + 0.5))


def test_branch_flips_locate_a_planted_change():
    """Oracle signatures of a state and of the same state with one cell changed: the
    flips are the faces and cells near that cell (the counting on the host is right)."""
    from hyperboliconvergence_gb300 import cases
    from hyperboliconvergence_gb300.solver import branch_flips
    rng = np.random.default_rng(3)
    mesh, bc, ref, q, sp = cases.quadrant_riemann(16, 12, rng)
    q = q * (1 + 0.02 * rng.standard_normal(q.shape))
    a = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux="ausmpup", limiter="minmod",
                               species=sp, ghost_ref=ref)
    a.set_state(q)
    s0 = a.face_signatures()
    assert branch_flips(s0, a.face_signatures())["faces"] == 0
    q2 = q.copy()
    q2[:, 7, 5] = q2[:, 7, 5] * np.array([-3.0, 3.0, 1.5, 1.5])
    a.set_state(q2)
    f = branch_flips(s0, a.face_signatures())
    assert f["faces"] > 0
    # a change in one cell reaches at most the faces of its 2-cell stencil
    si = s0[0] != a.face_signatures()[0]
    idx = np.argwhere(si)
    assert np.all(np.abs(idx[:, 0] - 7.5) <= 3) and np.all(np.abs(idx[:, 1] - 5) <= 2)
