"""Fast-time binning and along-track window culling (float64 oracle).

Restates soundersim ``kernels/geometry.py``. These are the integer decisions
that must agree bit-for-bit between the GPU path and the oracle.
"""

import numpy as np


def twtt_bin(twtt, t0, dt):
    """floor((twtt - t0) / dt) as int32 (geometry.py:18-24): pre-window times
    go negative instead of truncating toward zero."""
    return np.floor((twtt - t0) / dt).astype(np.int32)


def window_reach_m(t0, dt, n_samples, c):
    """Horizontal radius past which no path can bin inside the window
    (geometry.py:40-45): c * t_end / 2 with two spare bins, a 1e-5 relative
    margin and one metre."""
    t_end = float(t0) + (float(n_samples) + 2.0) * float(dt)
    return 0.5 * float(c) * t_end * (1.0 + 1e-5) + 1.0


def along_track_order(positions, centers):
    """Track axis, stable facet sort along it, and both projections
    (geometry.py:48-60). The axis is the horizontal first->last position
    direction, or +x when the track is a single point."""
    pos = np.asarray(positions, np.float64)
    a = pos[-1, :2] - pos[0, :2]
    length = np.linalg.norm(a)
    axis = a / length if length > 0 else np.array([1.0, 0.0])
    s_facet = np.asarray(centers, np.float64)[:, :2] @ axis
    order = np.argsort(s_facet, kind="stable")
    return order, pos[:, :2] @ axis, s_facet[order]


def block_windows(s_sorted, s_trace, reach, block_size, n_blocks):
    """Per-trace first block and the shared window length (geometry.py:63-78)
    covering every facet with |s_f - s_t| <= reach."""
    if not np.isfinite(reach):
        return np.zeros(len(s_trace), np.int32), int(n_blocks)
    first = np.searchsorted(s_sorted, s_trace - reach, "left")
    last = np.searchsorted(s_sorted, s_trace + reach, "right")
    b_first = first // block_size
    b_end = np.minimum(-(-last // block_size), n_blocks)
    n_win = int(max(1, int((b_end - b_first).max())))
    off = np.minimum(b_first, n_blocks - n_win)
    return off.astype(np.int32), n_win


def auto_block_size(n_traces, target_pairs, lo=512, hi=16384):
    """Power-of-two block size holding ~target_pairs lanes per step
    (geometry.py:81-90)."""
    ratio = max(target_pairs / max(int(n_traces), 1), 1.0)
    return int(np.clip(1 << int(round(np.log2(ratio))), lo, hi))


def culling_plan(positions, centers, *, t0, dt, n_samples, c, block_size,
                 target_pairs, window_cull=True):
    """Facet order, block size/count and per-trace windows exactly as the
    reference kernels derive them (coherent.py:284-296,
    multilayer.py:684-697). Returns (order, block_size, n_blocks, off,
    n_win)."""
    n = len(centers)
    bs = min(block_size or auto_block_size(len(positions), target_pairs), n)
    n_blocks = -(-n // bs)
    order, s_t, s_sorted = along_track_order(positions, centers)
    reach = window_reach_m(t0, dt, n_samples, c) if window_cull else np.inf
    off, n_win = block_windows(s_sorted, s_t, reach, bs, n_blocks)
    return order, bs, n_blocks, off, n_win
