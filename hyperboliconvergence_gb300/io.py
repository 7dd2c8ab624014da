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
* ``save_checkpoint`` / ``load_checkpoint``: a binary snapshot (HCCK format 2: a
  JSON header with the run's configuration, step, time and dt, float64 SoA arrays
  and a CRC-32) from which a run resumes bit for bit; a corrupted file is refused.
  The reference has no checkpoint (its only output is the result.dat above).

States are primitive {u, v, rho, p} arrays of shape (4, ni, nj).
"""
from __future__ import annotations

import json
import math
import os
import struct
import zlib

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


# ---------------------------------------------------------------- binary checkpoint
#
# Layout (little-endian), "HCCK" format 2:
#   8 bytes   magic b"HCCKPT\x00\x02"
#   u64       H, the byte length of the header
#   u64       P, the byte length of the payload
#   H bytes   header: UTF-8 JSON -- the run's configuration (law, basis, precision,
#             flux, limiter, RK table, dt mode, CFL, species, AUSM+up low-Mach settings,
#             corrections, tile), the mesh kind and shape, the boundary types, the step
#             count, the accumulated time t and the last step's dt, and one entry per
#             array {name, shape, offset} (offsets into the payload, 8-byte aligned)
#   P bytes   payload: the arrays as float64 -- mesh nodes, the boundary reference
#             layers that exist, the state in the solution basis (SoA planes)
#   u32       CRC-32 of every byte before it
# A file whose magic, lengths, CRC, header or array bounds do not check out is refused
# with CheckpointError; nothing is built from it.

MAGIC = b"HCCKPT\x00\x02"
_PRE = struct.Struct("<8sQQ")


class CheckpointError(ValueError):
    """A checkpoint file that is not a complete, intact HCCK file."""


def write_checkpoint(path, meta: dict, arrays: dict) -> None:
    """Write meta (JSON-serialisable) and float64 arrays as one HCCK file, atomically (a
    temporary file in the same directory, renamed over `path`)."""
    entries, chunks, off = [], [], 0
    for name, a in arrays.items():
        a = np.ascontiguousarray(a, dtype="<f8")
        entries.append({"name": name, "shape": list(a.shape), "offset": off})
        chunks.append(a.tobytes())
        off += a.nbytes
    header = json.dumps(dict(meta, arrays=entries), sort_keys=True).encode()
    body = _PRE.pack(MAGIC, len(header), off) + header + b"".join(chunks)
    crc = zlib.crc32(body) & 0xFFFFFFFF
    path = os.fspath(path)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as f:
        f.write(body)
        f.write(struct.pack("<I", crc))
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def read_checkpoint(path):
    """(meta, arrays) of an HCCK file, after checking its magic, lengths and CRC-32."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < _PRE.size + 4:
        raise CheckpointError("checkpoint truncated: shorter than its preamble")
    magic, hlen, plen = _PRE.unpack_from(data, 0)
    if magic != MAGIC:
        raise CheckpointError("not an HCCK format-2 checkpoint (bad magic)")
    if _PRE.size + hlen + plen + 4 != len(data):
        raise CheckpointError(f"checkpoint truncated or padded: {len(data)} bytes, the preamble says "
                              f"{_PRE.size + hlen + plen + 4}")
    body, (crc,) = data[:-4], struct.unpack("<I", data[-4:])
    if zlib.crc32(body) & 0xFFFFFFFF != crc:
        raise CheckpointError("checkpoint corrupted: CRC-32 mismatch")
    try:
        meta = json.loads(body[_PRE.size:_PRE.size + hlen].decode())
    except (UnicodeDecodeError, json.JSONDecodeError) as e:
        raise CheckpointError(f"checkpoint header unreadable: {e}") from e
    payload = body[_PRE.size + hlen:]
    arrays = {}
    for e in meta.pop("arrays", []):
        n = int(np.prod(e["shape"], dtype=np.int64))
        lo, hi = int(e["offset"]), int(e["offset"]) + 8 * n
        if lo < 0 or hi > len(payload) or lo % 8:
            raise CheckpointError(f"array {e['name']} lies outside the payload")
        arrays[e["name"]] = np.frombuffer(payload[lo:hi], dtype="<f8").reshape(e["shape"]).astype(np.float64)
    return meta, arrays


def save_checkpoint(path, solver) -> None:
    """Everything needed to resume a Solver's run bit for bit: mesh, boundary types and
    reference layers, species, configuration, the current state, the step count and the
    accumulated time (HCCK format 2, above)."""
    st = solver.sync()
    m = solver.mesh
    meta = {"format": 2, "law": solver.law, "basis": solver.basis, "precision": solver.precision,
            "flux": str(solver.flux), "limiter": str(solver.limiter), "rk": str(solver.rk), "dt_mode": solver.dt,
            "cfl": solver.cfl, "species": list(solver.species), "low_mach": solver.low_mach,
            "corrections": int(solver.corrections), "tile": solver.tile,
            "mesh": {"dims": 1 if getattr(m, "one_d", False) else 2, "ni": m.ni, "nj": m.nj},
            "nv": solver.nv, "bc": [str(b) for b in solver.bc], "step": int(solver.steps_done),
            "t": float(st.t), "dt": float(st.dt)}
    arrays = {"nodes": m.nodes, "state": solver.get_state()}
    for k, r in enumerate(solver.ref):
        if r is not None:
            arrays[f"ref{k}"] = r
    write_checkpoint(path, meta, arrays)


def load_checkpoint(path, stream=None):
    """A Solver rebuilt from an HCCK checkpoint: configuration, mesh, boundaries, state,
    step count and time restored.  A corrupted or truncated file raises CheckpointError
    before any device work."""
    from .solver import Mesh, Mesh1D, Solver
    meta, arrays = read_checkpoint(path)
    if meta.get("format") != 2:
        raise CheckpointError(f"unsupported checkpoint format {meta.get('format')!r}")
    mk = meta["mesh"]
    mesh = Mesh1D(arrays["nodes"]) if mk["dims"] == 1 else Mesh(arrays["nodes"])
    if (mesh.ni, mesh.nj) != (mk["ni"], mk["nj"]):
        raise CheckpointError("mesh nodes do not match the recorded shape")
    state = arrays["state"]
    want = (meta["nv"], mesh.ni) if mk["dims"] == 1 else (meta["nv"], mesh.ni, mesh.nj)
    if tuple(state.shape) != want:
        raise CheckpointError(f"state of shape {tuple(state.shape)}, expected {want}")
    nsides = 2 if mk["dims"] == 1 else 4
    ref = [arrays.get(f"ref{k}") for k in range(nsides)]
    s = Solver(mesh, meta["bc"][:nsides], None if all(r is None for r in ref) else ref, flux=meta["flux"],
               limiter=meta["limiter"], rk=meta["rk"], precision=meta["precision"], dt=meta["dt_mode"],
               cfl=meta["cfl"], species=tuple(meta["species"]), stream=stream, law=meta["law"],
               low_mach=None if meta["low_mach"] is None else tuple(meta["low_mach"]), basis=meta["basis"],
               tile=meta["tile"], corrections=meta["corrections"])
    s.set_state(state)
    s.set_time(meta["t"], meta["step"])
    return s
