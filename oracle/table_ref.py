"""CPU oracle of the flow's training-table generator (ntp_make_table).

TEST INFRASTRUCTURE ONLY: imported by tests/ to verify the table
kernels, never by the product path.

Restates, for hits already propagated and weighted: the PMT assignment of a
rotated module (check_pmt_hit, detection.jl:72-104 of chrhck/NeutrinoTelescopes,
with the FP32 cosine rule of the kernels), the per-(simulation, orientation,
PMT) sums of resample_simulation (pmt_frontend/pipeline.jl:86-116), the
Efraimidis-Spirakis selection keys (Philox4x32-10 keyed by the pair), the
time residual of calc_time_residual! (photon_prop_cuda.jl:906-924) and the
group features.  Plain numpy / Python loops: small cases only.
"""
from __future__ import annotations

import math

import numpy as np

TABLE_KEY = 0x54424C00
C_VAC = 0.299792458


def module_axes(pmt_coords: np.ndarray) -> np.ndarray:
    """Module-frame PMT axes [P x 3] from (theta, phi) columns, in float32
    trigonometry as the library computes them."""
    th = pmt_coords[0].astype(np.float32)
    ph = pmt_coords[1].astype(np.float32)
    return np.stack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)], -1).astype(np.float64)


def lab_axes(orientations: np.ndarray, pm: np.ndarray) -> np.ndarray:
    """[S*R x P x 3]: O . a for every orientation."""
    return np.einsum("nij,pj->npi", orientations, pm)


def group_features(src_pos, src_dir, log10_e, orientations, pm, R: int) -> np.ndarray:
    S = len(src_pos)
    P = len(pm)
    out = np.zeros((S * R * P, 5))
    ax = lab_axes(orientations, pm).reshape(S, R, P, 3)
    for s in range(S):
        p = np.asarray(src_pos[s], np.float64)
        d = np.linalg.norm(p)
        u = p / d
        v = np.asarray(src_dir[s], np.float64)
        vu = v @ u
        e1 = v - vu * u
        for r in range(R):
            for j in range(P):
                a = ax[s, r, j]
                au = a @ u
                e2 = a - au * u
                phi = math.atan2(np.cross(e1, e2) @ u, e1 @ e2)
                if phi < 0:
                    phi += 2 * math.pi
                out[(s * R + r) * P + j] = [2 * math.log(d) / math.log(200.0) - 1, vu, au, phi / math.pi - 1,
                                            (float(np.float32(log10_e[s])) - 4) / 2]
    return out


def assign_pairs(positions, source_index, orientations, pm, R: int, cos_open: float):
    """(hit index, group) of every (hit, orientation) pair with a PMT."""
    P = len(pm)
    ax = lab_axes(orientations, pm).astype(np.float32)
    pairs = []
    pos = positions.astype(np.float32)
    nrm = pos / np.sqrt((pos.astype(np.float64) ** 2).sum(1))[:, None].astype(np.float32)
    for i in range(len(pos)):
        s = int(source_index[i])
        for r in range(R):
            a = ax[s * R + r]
            dp = (a.astype(np.float64) @ nrm[i].astype(np.float64))
            hit = np.nonzero(dp > cos_open)[0]
            if hit.size:
                pairs.append((i, (s * R + r) * P + int(hit[0])))
    return pairs


def u01_53(a: int, b: int) -> float:
    m = ((a << 21) ^ (b >> 11)) & ((1 << 53) - 1)
    return (m + 0.5) / 9007199254740992.0


def pair_key(philox, photon_index: int, source_index: int, r: int, w: float, seed: int) -> float:
    ctr = (TABLE_KEY + r, photon_index & 0xFFFFFFFF, photon_index >> 32, source_index)
    key = (seed & 0xFFFFFFFF, seed >> 32)
    x = philox(ctr, key)
    return math.log(u01_53(x[0], x[1])) / w


def rows_wanted(n_drawn: int, n_pos: int, max_rows: int, wsum: float, w2sum: float) -> int:
    """Rows drawn from a group: min(N, hits with w > 0, max_rows, ESS/4 + 1)
    with ESS = (sum w)^2 / sum w^2."""
    ess = wsum * wsum / w2sum if w2sum > 0 else 0.0
    return min(n_drawn, n_pos, max_rows, int(ess / 4.0) + 1)


def select(keys: list[tuple[float, int]], want: int) -> set[int]:
    """The hit indices with the `want` largest keys."""
    return {i for _, i in sorted(keys, reverse=True)[:want]}
