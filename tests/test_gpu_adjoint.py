"""Discrete adjoint: gradients against central finite differences (h = 1e-6,
relative agreement 1e-6) for every differentiated limiter and the hand-reversed fluxes,
against the dual-number FP64 reference for every Euler flux the adjoint takes,
checkpointed versus fully stored reversal, fixed-ghost reference gradients, and
the torch.autograd.Function for dJ/dMach, dJ/dalpha and dJ/dq0."""
import math

import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Mesh, Solver

pytestmark = pytest.mark.gpu

H = 1e-6
GAMMA = 1.4


def cylinder_case(nr=10, nth=32, mach=0.4, seed=0):
    """Cylinder at 0.1 rad incidence from a smooth start whose every variable has
    gradients of order 1e-2 per unit length: limiter arguments then sit away from
    the kinks (a = 0, b = 0, a*b = 0) that central differences cannot resolve,
    except on a few zero-crossing curves."""
    mesh = Mesh.cylinder(nr, nth, 0.5, 4.0, 1.05)
    alpha = 0.1
    qinf = np.array([mach * math.cos(alpha), mach * math.sin(alpha), 1.0, 1.0 / GAMMA])
    rng = np.random.default_rng(seed)
    c = mesh.centres()
    bump = np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2))
    amp = np.array([0.02, 0.02, 0.03, 0.02]) * (1 + 0.2 * rng.random(4))
    shape = 0.5 * bump + 0.1 * c[0] + 0.07 * c[1]
    q = qinf[:, None, None] + amp[:, None, None] * shape[None]
    ref = [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None]
    return mesh, ["wall", "fixed", "periodic", "periodic"], ref, q


def make(case, flux="roe", limiter="vanalbada", rk="ssp34"):
    mesh, bc, ref, q = case
    s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk=rk, precision="fp64", dt="global", cfl=0.5,
               species=(GAMMA, 287.058, 0.4))
    s.set_state(q)
    return s


def fd_check(s, q0, nsteps, kind, kw, seed=1, direction=None):
    """Central difference of J along `direction` (default: seeded noise) against <g, d>."""
    J, g, refb, rates, st = s.gradient(nsteps, snapshots=3, kind=kind, **kw)
    rng = np.random.default_rng(seed)
    d = direction if direction is not None else \
        rng.standard_normal(q0.shape) * np.abs(q0).max(axis=(1, 2), keepdims=True) * 1e-2
    s.set_state(q0 + H * d)
    jp, _ = s.objective(nsteps, kind=kind, rates=rates, **kw)
    s.set_state(q0 - H * d)
    jm, _ = s.objective(nsteps, kind=kind, rates=rates, **kw)
    s.set_state(q0)
    fd = (jp - jm) / (2 * H)
    ad = float(np.sum(g * d))
    return J, fd, ad, st


@pytest.mark.parametrize("flux,limiter,rk", [
    ("roe", "nolimit1", "ssp11"), ("roe", "nolimit2", "ssp34"), ("rusanov", "nolimit3", "ssp33"),
    ("roe", "vanalbada", "ssp34"), ("roe", "vanleer", "ssp22"), ("rusanov", "minmod", "ssp33")])
def test_drag_gradient_matches_central_fd(flux, limiter, rk):
    """Direction d = q0 - far-field state: it scales the limiter arguments instead of
    adding noise to them, so no argument crosses a limiter kink (a = 0, b = 0, a = b)
    inside +/-h and the central difference resolves the derivative.  (Along seeded
    noise the kinked limiters' differences move with h by up to 1e-2: arguments near
    an extremum flip branch.)"""
    case = cylinder_case()
    s = make(case, flux, limiter, rk)
    d = case[3] - case[2][1][:, :1, None]
    J, fd, ad, st = fd_check(s, case[3], 12, "drag", {"scale": 1.0 / (0.5 * 0.4 ** 2 * 1.0)}, direction=d)
    assert np.isfinite(J) and abs(ad) > 0
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)
    assert st.adjoint_steps == 12


@pytest.mark.parametrize("flux,limiter,rk", [("roe", "nolimit2", "ssp34"), ("rusanov", "nolimit3", "ssp33")])
def test_drag_gradient_noise_direction(flux, limiter, rk):
    """Smooth reconstructions along an arbitrary (seeded noise) direction."""
    case = cylinder_case()
    s = make(case, flux, limiter, rk)
    J, fd, ad, st = fd_check(s, case[3], 12, "drag", {"scale": 1.0 / (0.5 * 0.4 ** 2 * 1.0)})
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_l2_gradient_on_periodic_vortex():
    mesh, bc, ref, q, sp = cases.isentropic_vortex(20)
    s = Solver(mesh, bc, ref, flux="rusanov", limiter="nolimit3", rk="ssp34", dt="global", species=sp)
    s.set_state(q)
    target = q * 0.98
    J, fd, ad, _ = fd_check(s, q, 8, "l2", {"target": target, "weight": (1.0, 1.0, 2.0, 1.0)})
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_checkpointed_equals_stored_reversal():
    case = cylinder_case(seed=4)
    s = make(case)
    kw = {"scale": 1.0}
    a = s.gradient(16, snapshots=2, kind="drag", **kw)
    b = s.gradient(16, snapshots=16, kind="drag", **kw)
    assert a[0] == b[0]
    assert np.array_equal(a[1], b[1])
    assert a[4].forward_steps > b[4].forward_steps


def test_reference_state_gradient_matches_fd():
    """Fixed-ghost reference states: an L2 objective over every cell, so the cells
    next to the far field carry the sensitivity (a wall-drag objective would see
    the far field only after the signal crossed the mesh)."""
    case = cylinder_case(seed=2)
    s = make(case, limiter="nolimit2")
    mesh, bc, ref, q = case
    kw = {"target": q * 0.98, "weight": (1.0, 1.0, 1.0, 1.0)}
    J, g, refb, rates, _ = s.gradient(10, snapshots=3, kind="l2", **kw)
    d = np.zeros_like(ref[1])
    d[0] = 0.01  # far-field u
    d[3] = 0.002  # far-field p
    s.set_bcs(bc, [None, ref[1] + H * d, None, None]); s.set_state(q)
    jp, _ = s.objective(10, kind="l2", rates=rates, **kw)
    s.set_bcs(bc, [None, ref[1] - H * d, None, None]); s.set_state(q)
    jm, _ = s.objective(10, kind="l2", rates=rates, **kw)
    fd = (jp - jm) / (2 * H)
    ad = float(np.sum(refb[1] * d))
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_autograd_mach_alpha():
    torch = pytest.importorskip("torch")
    from hyperboliconvergence_gb300.autograd import freestream, run_objective
    nr, nth, n = 10, 32, 10
    mesh = Mesh.cylinder(nr, nth, 0.5, 4.0, 1.05)
    s = Solver(mesh, ["wall", "fixed", "periodic", "periodic"],
               [None, np.zeros((4, nth)), None, None], flux="roe", limiter="vanalbada", dt="global",
               species=(GAMMA, 287.058, 0.4))

    def J_of(m, a, rates=None):
        qinf = freestream(m, a)
        q0 = qinf[:, None, None].expand(4, nr, nth).contiguous()
        ref1 = qinf[:, None].expand(4, nth).contiguous()
        cd = run_objective(s, q0, [None, ref1, None, None], n, snapshots=4, kind="drag",
                           scale=1.0, direction=(1.0, 0.0))
        return cd / (0.5 * m * m * 1.0)

    m = torch.tensor(0.4, dtype=torch.float64, requires_grad=True)
    a = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    J = J_of(m, a)
    J.backward()
    # finite differences at frozen timesteps: replay the forward run's rates
    qinf = freestream(m.detach(), a.detach()).numpy()
    s.set_bcs(s.bc, [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None])
    s.set_state(np.broadcast_to(qinf[:, None, None], (4, nr, nth)).copy())
    _, rates = s.objective(n, kind="drag", scale=1.0)

    def J_np(mv, av):
        q = np.array([mv * math.cos(av), mv * math.sin(av), 1.0, 1.0 / GAMMA])
        s.set_bcs(s.bc, [None, np.broadcast_to(q[:, None], (4, nth)).copy(), None, None])
        s.set_state(np.broadcast_to(q[:, None, None], (4, nr, nth)).copy())
        j, _ = s.objective(n, kind="drag", rates=rates, scale=1.0)
        return j / (0.5 * mv * mv)

    fdm = (J_np(0.4 + H, 0.05) - J_np(0.4 - H, 0.05)) / (2 * H)
    fda = (J_np(0.4, 0.05 + H) - J_np(0.4, 0.05 - H)) / (2 * H)
    assert abs(m.grad.item() - fdm) <= 1e-6 * abs(fdm), (m.grad.item(), fdm)
    assert abs(a.grad.item() - fda) <= 1e-6 * max(abs(fda), 1e-12), (a.grad.item(), fda)


def test_unsupported_configuration_is_reported():
    from hyperboliconvergence_gb300 import HCError
    case = cylinder_case()
    s = make(case, flux="central")
    with pytest.raises(HCError) as e:
        s.gradient(2, snapshots=1, kind="drag", scale=1.0)
    assert e.value.code == 5


@pytest.mark.parametrize("flux,limiter,rk,kind", [
    ("roe", "nolimit2", "ssp34", "drag"), ("roe", "vanalbada", "ssp34", "drag"), ("roe", "vanleer", "ssp22", "drag"),
    ("rusanov", "minmod", "ssp33", "drag"), ("roe", "nolimit1", "ssp11", "l2"), ("rusanov", "vanalbada", "ssp34", "l2"),
    # fluxes reversed by tangents (hc_tangent.cuh)
    ("slau", "vanalbada", "ssp34", "drag"), ("slau_ref", "minmod", "ssp33", "l2"), ("ausmpup", "vanleer", "ssp34", "drag"),
    ("ausmpup", "nolimit1", "ssp22", "l2"), ("roe_ws", "vanalbada", "ssp34", "drag"), ("roe_ws", "nolimit3", "ssp34", "l2")])
def test_gradient_matches_fp64_reference(flux, limiter, rk, kind):
    """<gradient, d> against the FP64 reference derivative: the CPU oracle run with
    forward-mode dual numbers (exact, timesteps frozen), along seeded noise in the
    initial state plus a far-field direction."""
    from oracle import oracle_py
    mesh, bc, ref, q = cylinder_case(nr=12, nth=32, seed=3)
    s = make((mesh, bc, ref, q), flux, limiter, rk)
    kw = {"scale": 2.0} if kind == "drag" else {"target": q * 0.98, "weight": (1.0, 0.5, 2.0, 1.0)}
    J, g, refb, rates, st = s.gradient(10, snapshots=3, kind=kind, **kw)
    rng = np.random.default_rng(11)
    dq = rng.standard_normal(q.shape) * 1e-2
    dref = [None, rng.standard_normal(ref[1].shape) * 1e-2, None, None]
    okw = dict(kind=kind, flux=flux, limiter=limiter, rk=rk, cfl=0.5, species=(GAMMA, 287.058, 0.4), ref=ref,
               dq0=dq, dref=dref)
    if kind == "drag":
        okw["scale"] = 2.0
    else:
        okw["target"], okw["weight"] = kw["target"], kw["weight"]
    Jo, dJo = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 10, **okw)
    ad = float(np.sum(g * dq) + np.sum(refb[1] * dref[1]))
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert abs(ad - dJo) <= 1e-9 * abs(dJo), (ad, dJo)


def test_fp32_adjoint_matches_fp64():
    """FP32 context: forward, recomputation and reverse sweep in FP32 (rates, timesteps
    and J in FP64) against the FP64 gradient on a Gaussian-sum instance, with a smooth
    reconstruction.  (With a limiter the two precisions can take different branches
    where the state is uniform up to round-off -- far from the Gaussians -- and the
    gradients there differ by O(1) of the local adjoint.)"""
    rng = np.random.default_rng(8)
    mesh, bc, ref, q, sp = cases.gaussian_sum(48, 40, rng, base=(0.5, 0.25, 5.0, 1.0))
    target = cases.gaussian_sum(48, 40, np.random.default_rng(9), base=(0.5, 0.25, 5.0, 1.0))[3]
    out = {}
    for prec in ("fp64", "fp32"):
        s = Solver(mesh, bc, ref, flux="rusanov", limiter="nolimit3", rk="ssp34", precision=prec, dt="global",
                   cfl=0.5, species=sp)
        s.set_state(q)
        J, g, refb, rates, st = s.gradient(20, snapshots=4, kind="l2", target=target)
        out[prec] = (J, g)
    (ja, ga), (jb, gb) = out["fp64"], out["fp32"]
    assert abs(jb - ja) <= 1e-5 * abs(ja)
    assert np.abs(gb - ga).max() <= 1e-3 * np.abs(ga).max()


@pytest.mark.parametrize("flux", ["slau", "ausmpup", "roe_ws"])
def test_tangent_flux_gradient_matches_central_fd(flux):
    """The tangent-reversed fluxes against central differences of the product's own objective."""
    case = cylinder_case(seed=4)
    s = make(case, flux=flux, limiter="vanalbada")
    q0 = case[3]
    direction = (q0 - np.array([0.4 * math.cos(0.1), 0.4 * math.sin(0.1), 1.0, 1.0 / GAMMA])[:, None, None])
    J, fd, ad, st = fd_check(s, q0, 6, "drag", {"scale": 3.0}, direction=direction)
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_tangent_flux_fp32_close_to_fp64():
    rng = np.random.default_rng(8)
    mesh, bc, ref, q, sp = cases.gaussian_sum(40, 36, rng, base=(0.5, 0.25, 5.0, 1.0))
    target = cases.gaussian_sum(40, 36, np.random.default_rng(9), base=(0.5, 0.25, 5.0, 1.0))[3]
    out = {}
    for prec in ("fp64", "fp32"):
        s = Solver(mesh, bc, ref, flux="slau", limiter="nolimit3", rk="ssp34", precision=prec, dt="global",
                   cfl=0.5, species=sp)
        s.set_state(q)
        out[prec] = s.gradient(10, snapshots=3, kind="l2", target=target)[:2]
    (ja, ga), (jb, gb) = out["fp64"], out["fp32"]
    assert abs(jb - ja) <= 1e-5 * abs(ja)
    assert np.abs(gb - ga).max() <= 1e-3 * np.abs(ga).max()


def test_double_float_adjoint_rejects_tangent_fluxes():
    from hyperboliconvergence_gb300 import HCError
    mesh, bc, ref, q = cylinder_case()
    s = Solver(mesh, bc, ref, flux="slau", limiter="vanalbada", precision="fp64_df", dt="global",
               species=(GAMMA, 287.058, 0.4))
    s.set_state(q)
    with pytest.raises(HCError, match="double-float"):
        s.gradient(2, snapshots=1, kind="drag", scale=1.0)


@pytest.mark.parametrize("bc1", ["riemann", "entropy"])
@pytest.mark.parametrize("flux,limiter,rk,kind", [("roe", "vanalbada", "ssp34", "drag"),
                                                  ("slau", "nolimit2", "ssp33", "l2"),
                                                  ("rusanov", "minmod", "ssp34", "l2")])
def test_farfield_gradient_matches_fp64_reference(bc1, flux, limiter, rk, kind):
    """Riemann-invariant and entropy far fields: the ghost update reversed by tangents,
    against the dual-number reference in the initial state and the far-field layer."""
    from oracle import oracle_py
    mesh, bc, ref, q = cylinder_case(nr=12, nth=32, seed=5)
    bc = ["wall", bc1, "periodic", "periodic"]
    s = make((mesh, bc, ref, q), flux, limiter, rk)
    kw = {"scale": 2.0} if kind == "drag" else {"target": q * 0.98, "weight": (1.0, 0.5, 2.0, 1.0)}
    J, g, refb, rates, st = s.gradient(10, snapshots=3, kind=kind, **kw)
    rng = np.random.default_rng(13)
    dq = rng.standard_normal(q.shape) * 1e-2
    dref = [None, rng.standard_normal(ref[1].shape) * 1e-2, None, None]
    okw = dict(kind=kind, flux=flux, limiter=limiter, rk=rk, cfl=0.5, species=(GAMMA, 287.058, 0.4), ref=ref,
               dq0=dq, dref=dref)
    if kind == "drag":
        okw["scale"] = 2.0
    else:
        okw["target"], okw["weight"] = kw["target"], kw["weight"]
    Jo, dJo = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 10, **okw)
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    ad = float(np.sum(g * dq) + np.sum(refb[1] * dref[1]))
    assert abs(ad - dJo) <= 1e-9 * abs(dJo), (ad, dJo)
    assert np.abs(refb[1]).max() > 0


def test_riemann_reference_gradient_matches_fd():
    case = cylinder_case(seed=2)
    mesh, _, ref, q = case
    bc = ["wall", "riemann", "periodic", "periodic"]
    s = make((mesh, bc, ref, q), limiter="nolimit2")
    kw = {"target": q * 0.98, "weight": (1.0, 1.0, 1.0, 1.0)}
    J, g, refb, rates, _ = s.gradient(10, snapshots=3, kind="l2", **kw)
    d = np.zeros_like(ref[1])
    d[0] = 0.01
    d[3] = 0.002
    s.set_bcs(bc, [None, ref[1] + H * d, None, None]); s.set_state(q)
    jp, _ = s.objective(10, kind="l2", rates=rates, **kw)
    s.set_bcs(bc, [None, ref[1] - H * d, None, None]); s.set_state(q)
    jm, _ = s.objective(10, kind="l2", rates=rates, **kw)
    fd = (jp - jm) / (2 * H)
    ad = float(np.sum(refb[1] * d))
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_double_float_adjoint_rejects_farfield():
    from hyperboliconvergence_gb300 import HCError
    mesh, _, ref, q = cylinder_case()
    s = Solver(mesh, ["wall", "riemann", "periodic", "periodic"], ref, flux="roe", limiter="vanalbada",
               precision="fp64_df", dt="global", species=(GAMMA, 287.058, 0.4))
    s.set_state(q)
    with pytest.raises(HCError, match="double-float"):
        s.gradient(2, snapshots=1, kind="drag", scale=1.0)
