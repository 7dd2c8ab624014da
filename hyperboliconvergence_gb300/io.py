"""Solution and mesh files in the reference drivers' gnuplot text layout, and a
binary checkpoint of a solver's state.

* ``write_mesh_dat``: mesh nodes "x y", one per line, a blank line after each
  i-row of nodes (cpp/script/euler/cylinder2D.cpp:236-266).
* ``write_cylinder_result_dat``: per cell "theta z r" then the state relative to
  the freestream -- (rho-rho0)/rho0, u/|U0|, v/|U0|, (p-p0)/p0, (s-s0)/s0, a/a0
  with s = a^2/(gamma rho^(gamma-1)) -- a blank line after each i-row
  (cylinder2D.cpp:35-63, 192-233).  The reference writes the radius of a
  uniformly spaced O-grid, rc + (i+0.5)dr; here it is the radius and angle of the
  cell centroid, which is the same point on a uniform grid and the true one on a
  stretched grid.
* ``write_cartesian_result_dat``: per cell "x y" of the centroid then rho/rho0,
  u, v, p-p0, s/s0, a/a0, |u|/a, a blank line after each i-row
  (cpp/script/euler/gresho2D.cpp:36-69, 226-265).
* ``save_checkpoint`` / ``load_checkpoint``: mesh nodes, boundary types and
  reference layers, species, configuration and the primitive state in one
  ``.npz`` file, enough to resume a run.

States are primitive {u, v, rho, p} arrays of shape (4, ni, nj).
"""
from __future__ import annotations

import math

import numpy as np


def _fmt(x: float, precision: int) -> str:
    return f"{x:.{precision}e}"


def _sound2(q, gamma):
    return gamma * q[3] / q[2]


def write_mesh_dat(path, mesh, precision: int = 8) -> None:
    nodes = mesh.nodes
    with open(path, "w") as f:
        for i in range(mesh.ni + 1):
            for j in range(mesh.nj + 1):
                f.write(f"{_fmt(nodes[i, j, 0], precision)} {_fmt(nodes[i, j, 1], precision)} \n")
            f.write("\n")


def write_cylinder_result_dat(path, mesh, q, qref, gamma: float = 1.4, precision: int = 8) -> None:
    q = np.asarray(q, dtype=np.float64)
    c = mesh.centres()
    r = np.hypot(c[0], c[1])
    th = np.mod(np.arctan2(c[1], c[0]), 2 * math.pi)
    a = np.sqrt(_sound2(q, gamma))
    s = a * a / (gamma * q[2] ** (gamma - 1))
    r0, p0 = qref[2], qref[3]
    u0 = math.hypot(qref[0], qref[1])
    a0 = math.sqrt(gamma * p0 / r0)
    s0 = a0 * a0 / (gamma * r0 ** (gamma - 1))
    cols = [(q[2] - r0) / r0, q[0] / u0, q[1] / u0, (q[3] - p0) / p0, (s - s0) / s0, a / a0]
    with open(path, "w") as f:
        for i in range(mesh.ni):
            for j in range(mesh.nj):
                head = f"{_fmt(th[i, j], precision)} {_fmt(0.0, precision)} {_fmt(r[i, j], precision)} "
                f.write(head + " ".join(_fmt(col[i, j], precision) for col in cols) + "\n")
            f.write("\n")


def write_cartesian_result_dat(path, mesh, q, qref, gamma: float = 1.4, precision: int = 16) -> None:
    q = np.asarray(q, dtype=np.float64)
    c = mesh.centres()
    a = np.sqrt(_sound2(q, gamma))
    s = a * a / (gamma * q[2] ** (gamma - 1))
    r0, p0 = qref[2], qref[3]
    a0 = math.sqrt(gamma * p0 / r0)
    s0 = a0 * a0 / (gamma * r0 ** (gamma - 1))
    speed = np.hypot(q[0], q[1])
    cols = [q[2] / r0, q[0], q[1], q[3] - p0, s / s0, a / a0, speed / a]
    with open(path, "w") as f:
        for i in range(mesh.ni):
            for j in range(mesh.nj):
                head = f"{_fmt(c[0][i, j], precision)} {_fmt(c[1][i, j], precision)} "
                f.write(head + " ".join(_fmt(col[i, j], precision) for col in cols) + "\n")
            f.write("\n")


def read_dat(path):
    """Blocks of a gnuplot text file: a list (one per i-row) of 2D arrays."""
    blocks, cur = [], []
    with open(path) as f:
        for line in f:
            if line.strip():
                cur.append([float(x) for x in line.split()])
            elif cur:
                blocks.append(np.array(cur))
                cur = []
    if cur:
        blocks.append(np.array(cur))
    return blocks


def save_checkpoint(path, solver) -> None:
    """Mesh, boundary set-up, species, configuration and current state of a Solver."""
    m = solver.mesh
    refs = {f"ref{k}": (np.zeros((0,)) if r is None else np.asarray(r, dtype=np.float64))
            for k, r in enumerate(solver.ref)}
    np.savez(path, format=np.array([1]), nodes=m.nodes,
             bc=np.array(solver.bc), species=np.array(solver.species, dtype=np.float64),
             config=np.array([str(solver.flux), str(solver.limiter), str(solver.rk), solver.precision,
                              solver.dt]),
             cfl=solver.cfl, state=solver.get_state(), **refs)


def load_checkpoint(path, stream=None):
    """A Solver rebuilt from a checkpoint, its state restored."""
    from .solver import Mesh, Solver
    d = np.load(path, allow_pickle=False)
    if int(d["format"][0]) != 1:
        raise ValueError("unknown checkpoint format")
    mesh = Mesh(d["nodes"])
    ref = [None if d[f"ref{k}"].size == 0 else d[f"ref{k}"] for k in range(4)]
    flux, limiter, rk, precision, dt = (str(x) for x in d["config"])
    s = Solver(mesh, [str(b) for b in d["bc"]], ref, flux=flux, limiter=limiter, rk=rk, precision=precision,
               dt=dt, cfl=float(d["cfl"]), species=tuple(float(x) for x in d["species"]), stream=stream)
    s.set_state(d["state"])
    return s
