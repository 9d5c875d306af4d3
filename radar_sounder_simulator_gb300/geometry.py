"""Host-side culling plan: along-track facet order and per-trace block
windows (soundersim ``kernels/geometry.py``).

These integer decisions decide which facets each trace sums, so they follow
the reference's rules exactly (stable argsort along the first->last track
axis, searchsorted windows padded by the reach rule, power-of-two block size)
and are checked bit-for-bit against the reference's own outputs in the
test-suite.
"""

from typing import NamedTuple

import numpy as np


def window_reach_m(t0, dt, n_samples, c):
    """Radius past which nothing bins inside the window (geometry.py:40-45)."""
    t_end = float(t0) + (float(n_samples) + 2.0) * float(dt)
    return 0.5 * float(c) * t_end * (1.0 + 1e-5) + 1.0


def auto_block_size(n_traces, target_pairs, lo=512, hi=16384):
    """Power-of-two facets per block (geometry.py:81-90)."""
    ratio = max(target_pairs / max(int(n_traces), 1), 1.0)
    return int(np.clip(1 << int(round(np.log2(ratio))), lo, hi))


class CullPlan(NamedTuple):
    order: np.ndarray      # (N,) facet permutation (stable along-track sort)
    block_size: int
    n_blocks: int
    off: np.ndarray        # (T,) int32 first block of each trace window
    n_win: int             # blocks per window


def cull_plan(positions, centers, *, t0, dt, n_samples, c, block_size,
              target_pairs, window_cull=True):
    """Order + windows as coherent.py:284-296 / multilayer.py:684-697."""
    pos = np.asarray(positions, np.float64)
    cen = np.asarray(centers, np.float64)
    n = len(cen)
    bs = min(block_size or auto_block_size(len(pos), target_pairs), n)
    n_blocks = -(-n // bs)
    d = pos[-1, :2] - pos[0, :2]
    nrm = np.linalg.norm(d)
    axis = d / nrm if nrm > 0 else np.array([1.0, 0.0])
    s_f = cen[:, :2] @ axis
    order = np.argsort(s_f, kind="stable")
    s_sorted = s_f[order]
    s_t = pos[:, :2] @ axis
    if not window_cull:
        return CullPlan(order, bs, n_blocks, np.zeros(len(pos), np.int32),
                        int(n_blocks))
    reach = window_reach_m(t0, dt, n_samples, c)
    lo = np.searchsorted(s_sorted, s_t - reach, "left")
    hi = np.searchsorted(s_sorted, s_t + reach, "right")
    b_lo = lo // bs
    b_hi = np.minimum(-(-hi // bs), n_blocks)
    n_win = int(max(1, int((b_hi - b_lo).max())))
    off = np.minimum(b_lo, n_blocks - n_win).astype(np.int32)
    return CullPlan(order, bs, n_blocks, off, n_win)
