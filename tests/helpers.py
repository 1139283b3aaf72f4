"""Shared helpers for the parity tests."""
from __future__ import annotations

import numpy as np


def defined_entries(scn) -> np.ndarray:
    """Boolean (Ng, Q): population entries whose value the reference defines after a step.

    Interior fluid cells and ghost cells without a handler: every direction. Cells bound to a
    handler: the directions that face an interior fluid cell (what boundary.hpp writes each
    step); their other directions only hold stale initial values.
    """
    q = scn.q
    vel = scn.model.velocities
    shape = (scn.zl + 2, scn.yl + 2, scn.xl + 2)
    nonfluid = np.zeros(shape, dtype=bool)
    for b in scn.boundaries:
        x0, xe, y0, ye, z0, ze = b.extent
        nonfluid[z0:ze + 1, y0:ye + 1, x0:xe + 1] = True
    if scn.solid is not None:
        nonfluid[1:-1, 1:-1, 1:-1] |= scn.solid != 0
    interior = np.zeros(shape, dtype=bool)
    interior[1:-1, 1:-1, 1:-1] = True
    ifluid = interior & ~nonfluid
    out = np.zeros(shape + (q,), dtype=bool)
    out[~nonfluid] = True
    for k in range(q):
        cx, cy, cz = vel[k]
        nb = np.zeros(shape, dtype=bool)
        src = ifluid
        # nb[z, y, x] = ifluid[z + cz, y + cy, x + cx] where in range
        zs = slice(max(0, -cz), shape[0] - max(0, cz))
        ys = slice(max(0, -cy), shape[1] - max(0, cy))
        xs = slice(max(0, -cx), shape[2] - max(0, cx))
        zd = slice(max(0, cz), shape[0] - max(0, -cz))
        yd = slice(max(0, cy), shape[1] - max(0, -cy))
        xd = slice(max(0, cx), shape[2] - max(0, -cx))
        nb[zs, ys, xs] = src[zd, yd, xd]
        out[..., k] |= nonfluid & nb
    if any(scn.periodic):
        # ghost planes of periodic axes carry no state
        if scn.periodic[0]:
            out[:, :, [0, -1]] = False
        if scn.periodic[1]:
            out[:, [0, -1], :] = False
        if scn.periodic[2]:
            out[[0, -1], :, :] = False
    return out.reshape(-1, q)


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def nonfluid_cells(scn) -> np.ndarray:
    """Boolean (Ng,): cells bound to a handler (boundary boxes and solid interior cells)."""
    shape = (scn.zl + 2, scn.yl + 2, scn.xl + 2)
    nonfluid = np.zeros(shape, dtype=bool)
    for b in scn.boundaries:
        x0, xe, y0, ye, z0, ze = b.extent
        nonfluid[z0:ze + 1, y0:ye + 1, x0:xe + 1] = True
    if scn.solid is not None:
        nonfluid[1:-1, 1:-1, 1:-1] |= scn.solid != 0
    return nonfluid.reshape(-1)


def linked_fluid_cells(scn) -> np.ndarray:
    """Boolean (zl, yl, xl): interior fluid cells with at least one non-fluid neighbour x + c_q
    (the cells whose pulls read handler values; non-periodic scenarios)."""
    shape = (scn.zl + 2, scn.yl + 2, scn.xl + 2)
    nonfluid = nonfluid_cells(scn).reshape(shape)
    out = np.zeros((scn.zl, scn.yl, scn.xl), dtype=bool)
    for cx, cy, cz in scn.model.velocities:
        out |= nonfluid[1 + cz:scn.zl + 1 + cz, 1 + cy:scn.yl + 1 + cy, 1 + cx:scn.xl + 1 + cx]
    return out & scn.fluid_mask_interior()


def precision_errors(scn, pops, rho, u, ref_pops, ref_rho, ref_u) -> dict:
    """Largest absolute errors of a reduced-precision run against the reference's FP64 result,
    split by where they arise: handler values (entries of non-fluid cells that a handler writes),
    fluid-cell populations, and density / velocity of the fluid cells next to a boundary
    ("linked") and of the other fluid cells ("bulk")."""
    mask = defined_entries(scn)
    nf = nonfluid_cells(scn)
    d = np.abs(pops - ref_pops)
    handler = mask & nf[:, None]
    fluid = mask & ~nf[:, None]
    linked = linked_fluid_cells(scn)
    bulk = scn.fluid_mask_interior() & ~linked
    du = np.abs(u - ref_u).max(axis=-1)
    dr = np.abs(rho - ref_rho)

    def mx(a, m):
        return float(a[m].max()) if m.any() else 0.0
    return {"handler_entries": mx(d, handler), "fluid_entries": mx(d, fluid),
            "u_linked": mx(du, linked), "u_bulk": mx(du, bulk),
            "rho_linked": mx(dr, linked), "rho_bulk": mx(dr, bulk),
            "n_handler_entries": int(handler.sum()), "n_linked": int(linked.sum())}
