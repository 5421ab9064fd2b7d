"""Shared definitions of the parity cases at the benchmark sizes.

The two generator workloads the headline numbers are quoted on are too large
to keep whole evaluations as fixtures (a 1024 x 1024 grid and 1.25 M gcells
are tens of MB per array), so the reference's results there are kept as
digests: SHA-256 of the integer and bit-exact arrays, norms of the float
arrays and their values at a fixed sample of indices.  make_golden_scale.py
writes them from the reference build; the tests recompute the same digests
from the GPU path (and compare the GPU with the oracle on the whole arrays).
"""

from __future__ import annotations

import hashlib

import numpy as np

# workload name -> generator seed (the seed bench.py uses)
SCALE_WORKLOADS = {
    "200k_cells_40macros_512bins": 1,
    "1m_cells_1024bins": 1,
}
EVAL_SEED = 7
N_SAMPLES = 8192


def eval_coords(core, drect, seed: int = EVAL_SEED) -> np.ndarray:
    """Seeded gcell centres that keep every density rectangle inside the
    core (one DBU of margin): x = lx + w/2 + 1 + U (core width - w - 2),
    evaluated in float64 and rounded to float32, x and y interleaved.
    `drect` is the gcells' (dLx, dLy, dUx, dUy) from any placement state."""
    drect = np.asarray(drect, np.int64).reshape(-1, 4)
    n = len(drect)
    rng = np.random.default_rng(seed)
    ux = rng.random(n)
    uy = rng.random(n)
    ddx = (drect[:, 2] - drect[:, 0]).astype(np.float64)
    ddy = (drect[:, 3] - drect[:, 1]).astype(np.float64)
    cdx = float(core[2] - core[0])
    cdy = float(core[3] - core[1])
    out = np.empty(2 * n, np.float32)
    out[0::2] = core[0] + ddx / 2 + 1 + ux * np.maximum(cdx - ddx - 2, 0.0)
    out[1::2] = core[1] + ddy / 2 + 1 + uy * np.maximum(cdy - ddy - 2, 0.0)
    return out


def sample_indices(n: int, k: int = N_SAMPLES, seed: int = 11) -> np.ndarray:
    """Sorted distinct indices into an array of n elements."""
    k = min(k, n)
    return np.sort(np.random.default_rng(seed).choice(n, size=k, replace=False))


def sha(a) -> str:
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes()).hexdigest()


def eval_digest(ev: dict, n_gcells: int, n_bins: int) -> dict:
    """Digest of one evaluation.  `ev` holds inst_area, filler_area,
    nonplace_area (int64), density, phi, ex, ey (float32, per bin) and
    wl_grad, density_grad (float32, x y per gcell)."""
    gi = sample_indices(n_gcells)
    bi = sample_indices(n_bins, seed=13)
    out = {}
    for k in ("inst_area", "filler_area", "nonplace_area"):
        a = np.asarray(ev[k], np.int64).ravel()
        out[k + "_sha"] = np.array(sha(a))
        out[k + "_sum"] = np.array(int(a.sum()), np.int64)
    out["density_sha"] = np.array(sha(np.asarray(ev["density"], np.float32).ravel()))
    for k in ("phi", "ex", "ey", "density"):
        a = np.asarray(ev[k], np.float32).ravel()
        out[k + "_norm"] = np.array(float(np.linalg.norm(a.astype(np.float64))))
        out[k + "_sample"] = a[bi]
    for k in ("wl_grad", "density_grad"):
        a = np.asarray(ev[k], np.float32).reshape(-1, 2)
        out[k + "_norm"] = np.array(float(np.linalg.norm(a.astype(np.float64))))
        out[k + "_sample"] = a[gi]
    out["gcell_index"] = gi.astype(np.int32)
    out["bin_index"] = bi.astype(np.int32)
    return out
