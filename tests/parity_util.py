"""Helpers comparing the engine's exports with the oracle's arrays.

The oracle keeps the reference layout (3 components per vector, 3x3 blocks,
also in 2D); the engine stores D components.  These helpers project the
oracle arrays onto the engine layout (the z parts of a 2D case are exact
zeros in the reference, see source/main.cpp:49 and 2284-2288)."""
from __future__ import annotations

import numpy as np

from mphimplicit_gb300 import casegen


def small_cases():
    """(name, dim, params, particles) of the parity cases."""
    out = []
    p, parts = casegen.square_drop_2d(scale=0.1, seed=0)
    out.append(("dam2d", 2, p, parts))
    # 2D with two fluid types, surface tension, asymmetric interaction ratios
    # and a moving, rotating type-3 wall (the top lid)
    l0 = 0.01
    def lid(wc):
        return np.where(wc[:, 1] >= 14, 3, 2)
    parts2 = casegen.dam_case(2, (10, 8), (16, 14), l0, seed=3, wall_type_fn=lid,
                              fluid_types=(np.arange(80) % 3 == 0).astype(np.int32))
    p2 = casegen.baseline_params(2, l0, 1.0e-4)
    p2.surface_tension = (0.072, 0.05, 0.0, 0.0)
    p2.density = (1000.0, 1200.0, 1000.0, 1000.0)
    p2.shear_viscosity = (0.1, 0.3, 0.1, 0.1)
    p2.interaction_ratio = ((1.0, 0.8, 1.0, 0.9), (0.8, 1.0, 0.7, 1.0), (1.0, 1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
    p2.wall3 = (0.08, 0.17, 0.0, 0.05, 0.0, 0.0, 0.0, 0.0, 2.0)
    out.append(("surface2d", 2, p2, parts2))
    parts3 = casegen.dam_case(3, (5, 5, 5), (8, 7, 7), 0.005, seed=0)
    p3 = casegen.baseline_params(3, 0.005, 5.0e-5)
    out.append(("cube3d", 3, p3, parts3))
    parts4 = casegen.dam_case(3, (4, 5, 4), (7, 7, 6), 0.005, seed=5,
                              fluid_types=(np.arange(80) % 2).astype(np.int32))
    p4 = casegen.baseline_params(3, 0.005, 5.0e-5)
    p4.surface_tension = (0.072, 0.072, 0.0, 0.0)
    p4.density = (1000.0, 1200.0, 1000.0, 1000.0)
    p4.wall2 = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    out.append(("surface3d", 3, p4, parts4))
    return out


def vec_proj(a: np.ndarray, dim: int) -> np.ndarray:
    return a.reshape(-1, 3)[:, :dim]


def rel(a, b) -> float:
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    s = np.max(np.abs(b)) if b.size else 0.0
    if s == 0.0:
        return float(np.max(np.abs(a))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / s)


def csr_blocks_oracle(ptr, val, nrow_particles, cnt, dim, per_block=True):
    """Oracle CSR (rows 3*i+r, entries (k, s) or k) -> flat list in engine
    order restricted to r, s < dim."""
    out = []
    for i in range(nrow_particles):
        for r in range(dim):
            base = ptr[3 * i + r]
            if per_block:
                blk = val[base: base + 3 * cnt[i]].reshape(cnt[i], 3)[:, :dim]
                out.append(blk.ravel())
            else:
                out.append(val[base: base + cnt[i]])
    return np.concatenate(out) if out else np.zeros(0)


def mg_proj(cof_oracle: np.ndarray, dim: int) -> np.ndarray:
    rows3, width3 = cof_oracle.shape
    cells, S = rows3 // 3, width3 // 3
    return cof_oracle.reshape(cells, 3, S, 3)[:, :dim, :, :dim].reshape(-1)
