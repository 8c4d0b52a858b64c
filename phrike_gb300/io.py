"""Solution snapshots and checkpoints in the reference's .npz layout.

save_solution_snapshot / load_checkpoint follow phrike/io.py:32-236: a file
``snapshot_t{t:.6f}[_{tag}].npz`` holding t, the conservative state U, the
grid coordinates, the primitive fields (rho, u / ux, uy, uz, p; MHD adds Bx,
By, Bz and div_b), a ``meta`` dict (grid sizes, lengths, gamma) and a
creation stamp.  The state is read back from the device once per snapshot;
the primitives written beside it are output formatting on the host copy.

``Snapshot`` is the in-memory form the serving loop uses to pause a resident
solve and resume it later (problem family, grid, time, end time, state).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from datetime import datetime, timezone
from typing import Any, Dict, Optional

import numpy as np


def _host(a: Any) -> np.ndarray:
    if hasattr(a, "detach"):
        return a.detach().to("cpu").double().numpy()
    return np.asarray(a, dtype=np.float64)


def _primitives(U: np.ndarray, gamma: float) -> Dict[str, np.ndarray]:
    """Primitive fields of the snapshot file (equations.py primitive())."""
    if U.shape[0] == 8:  # MHD [rho, m(3), E, B(3)]
        rho = U[0]
        ux, uy, uz = U[1] / rho, U[2] / rho, U[3] / rho
        Bx, By, Bz = U[5], U[6], U[7]
        p = (gamma - 1.0) * (U[4] - 0.5 * rho * (ux * ux + uy * uy + uz * uz) - 0.5 * (Bx * Bx + By * By + Bz * Bz))
        return dict(rho=rho, ux=ux, uy=uy, uz=uz, p=p, Bx=Bx, By=By, Bz=Bz)
    nd = U.shape[0] - 2
    rho = U[0]
    vel = [U[1 + a] / rho for a in range(nd)]
    p = (gamma - 1.0) * (U[nd + 1] - 0.5 * rho * sum(v * v for v in vel))
    if nd == 1:
        return dict(rho=rho, u=vel[0], p=p)
    names = ["ux", "uy", "uz"][:nd]
    return dict(rho=rho, p=p, **dict(zip(names, vel)))


def save_solution_snapshot(outdir: str, t: float, U: Any, grid: Any, equations: Any, tag: Optional[str] = None,
                           tracers: Any = None) -> str:
    """Write one snapshot (phrike/io.py:103-236) and return its path; with
    tracers, their positions and mass as tracer_x/y/z and tracer_mass
    (io.py:86-100)."""
    os.makedirs(outdir, exist_ok=True)
    ts = f"t{t:.6f}"
    if tag:
        ts = f"{ts}_{tag}"
    path = os.path.join(outdir, f"snapshot_{ts}.npz")
    Uh = _host(U)
    gamma = float(equations.gamma)
    nd = len(Uh.shape) - 1
    prim = _primitives(Uh, gamma)
    coords = {"x": _host(grid.x)}
    meta: Dict[str, Any]
    if nd == 3:
        coords.update(y=_host(grid.y), z=_host(grid.z))
        meta = {"Nx": grid.Nx, "Ny": grid.Ny, "Nz": grid.Nz, "Lx": grid.Lx, "Ly": grid.Ly, "Lz": grid.Lz,
                "gamma": gamma}
    elif nd == 2:
        coords.update(y=_host(grid.y))
        meta = {"Nx": grid.Nx, "Ny": grid.Ny, "Lx": grid.Lx, "Ly": grid.Ly, "gamma": gamma}
    else:
        meta = {"N": grid.N, "Lx": grid.Lx, "gamma": gamma}
    extra = {}
    if Uh.shape[0] == 8:
        meta = dict(meta, mhd=True)
        if nd == 2 and hasattr(grid, "divergence"):
            try:
                extra["div_b"] = _host(grid.divergence(U[5], U[6]))
            except Exception:
                pass
    if tracers is not None:
        extra["tracer_x"] = _host(tracers.x)
        for k in ("y", "z"):
            if hasattr(tracers, k):
                extra[f"tracer_{k}"] = _host(getattr(tracers, k))
        if hasattr(tracers, "mass"):
            extra["tracer_mass"] = np.asarray(tracers.mass)
    np.savez(path, t=t, U=Uh, meta=meta, created=str(datetime.now(timezone.utc).replace(tzinfo=None)),
             **coords, **prim, **extra)
    return path


def load_checkpoint(checkpoint_path: str) -> Dict[str, Any]:
    """Read a snapshot back (phrike/io.py:32-85): t, U, meta, coordinates and
    the primitive fields."""
    if not os.path.exists(checkpoint_path):
        raise FileNotFoundError(f"Checkpoint file not found: {checkpoint_path}")
    data = np.load(checkpoint_path, allow_pickle=True)
    out: Dict[str, Any] = {"t": float(data["t"]), "U": data["U"],
                           "meta": data["meta"].item() if "meta" in data else {}}
    for k in ("x", "y", "z"):
        if k in data:
            out[k] = data[k]
    out["primitive_vars"] = {k: data[k] for k in ("rho", "u", "ux", "uy", "uz", "p") if k in data}
    for k in ("tracer_x", "tracer_y", "tracer_z", "tracer_mass"):
        if k in data:
            out[k] = data[k]
    return out


@dataclass
class Snapshot:
    """A paused solve: problem family, points per axis, time, end time and
    the conservative state (host copy, float32 as resident on the device)."""

    family: str
    n: int
    t: float
    t_end: float
    U: np.ndarray
    params: Dict = field(default_factory=dict)

    def save(self, path: str) -> str:
        np.savez(path, t=self.t, t_end=self.t_end, U=self.U,
                 meta={"family": self.family, "n": self.n, "params": self.params})
        return path

    @staticmethod
    def load(path: str) -> "Snapshot":
        d = np.load(path, allow_pickle=True)
        m = d["meta"].item()
        return Snapshot(m["family"], int(m["n"]), float(d["t"]), float(d["t_end"]), d["U"], dict(m["params"]))
