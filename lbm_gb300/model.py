"""Lattice models D3Q15 / D3Q19 / D3Q27 (host-side tables).

Same velocity orderings and weights as the reference's lbm::model structs (model.h:13-139) and as
the device tables in csrc/lattice.cuh; the opposite of q is Q-1-q (model.h:36-39).
"""
from __future__ import annotations

import numpy as np

# lbmdefinitions.h:47 -- 0.57735026919l converted to double
C_S = float.fromhex("0x1.279a745904047p-1")


class _Model:
    def __init__(self, name: str, velocities, weights):
        self.name = name
        self.D = 3
        self.velocities = np.array(velocities, dtype=np.int64)
        self.Q = len(self.velocities)
        self.weights = np.array(weights, dtype=np.float64)

    def inv(self, q: int) -> int:
        return self.Q - 1 - q

    def velocity_index(self, u: int, v: int, w: int) -> int:
        for q, c in enumerate(self.velocities):
            if tuple(c) == (u, v, w):
                return q
        raise ValueError(f"{(u, v, w)} is not a {self.name} velocity")

    def feq(self, rho, u):
        """Equilibrium of collision.hpp:33-51 for arrays rho[...] and u[..., 3] -> [..., Q]."""
        rho = np.asarray(rho, dtype=np.float64)
        u = np.asarray(u, dtype=np.float64)
        cu = np.einsum("qd,...d->...q", self.velocities.astype(np.float64), u)
        uu = np.sum(u * u, axis=-1)[..., None]
        return self.weights * rho[..., None] * (1 + cu / (C_S * C_S) + cu * cu / (2 * C_S * C_S * C_S * C_S)
                                                - uu / (2 * C_S * C_S))

    def __repr__(self) -> str:
        return f"lbm_gb300.model.{self.name.lower()}"


d3q15 = _Model("D3Q15",
               [(-1, -1, -1), (1, -1, -1), (0, 0, -1), (-1, 1, -1), (1, 1, -1),
                (0, -1, 0), (-1, 0, 0), (0, 0, 0), (1, 0, 0), (0, 1, 0),
                (-1, -1, 1), (1, -1, 1), (0, 0, 1), (-1, 1, 1), (1, 1, 1)],
               [1 / 72, 1 / 72, 8 / 72, 1 / 72, 1 / 72, 8 / 72, 8 / 72, 16 / 72, 8 / 72, 8 / 72,
                1 / 72, 1 / 72, 8 / 72, 1 / 72, 1 / 72])
d3q19 = _Model("D3Q19",
               [(0, -1, -1), (-1, 0, -1), (0, 0, -1), (1, 0, -1), (0, 1, -1),
                (-1, -1, 0), (0, -1, 0), (1, -1, 0), (-1, 0, 0), (0, 0, 0),
                (1, 0, 0), (-1, 1, 0), (0, 1, 0), (1, 1, 0), (0, -1, 1),
                (-1, 0, 1), (0, 0, 1), (1, 0, 1), (0, 1, 1)],
               [1 / 36, 1 / 36, 2 / 36, 1 / 36, 1 / 36, 1 / 36, 2 / 36, 1 / 36, 2 / 36, 12 / 36,
                2 / 36, 1 / 36, 2 / 36, 1 / 36, 1 / 36, 1 / 36, 2 / 36, 1 / 36, 1 / 36])
d3q27 = _Model("D3Q27",
               [(q % 3 - 1, (q // 3) % 3 - 1, q // 9 - 1) for q in range(27)],
               [(1, 4, 1, 4, 16, 4, 1, 4, 1, 4, 16, 4, 16, 64, 16, 4, 16, 4, 1, 4, 1, 4, 16, 4, 1, 4, 1)[q] / 216
                for q in range(27)])

MODELS = {15: d3q15, 19: d3q19, 27: d3q27}


def get(q) -> _Model:
    if isinstance(q, _Model):
        return q
    return MODELS[int(q)]
