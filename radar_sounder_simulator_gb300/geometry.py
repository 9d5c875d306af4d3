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
import torch


def window_reach_m(t0, dt, n_samples, c):
    """Radius past which nothing bins inside the window (geometry.py:40-45)."""
    t_end = float(t0) + (float(n_samples) + 2.0) * float(dt)
    return 0.5 * float(c) * t_end * (1.0 + 1e-5) + 1.0


def auto_block_size(n_traces, target_pairs, lo=512, hi=16384):
    """Power-of-two facets per block (geometry.py:81-90)."""
    ratio = max(target_pairs / max(int(n_traces), 1), 1.0)
    return int(np.clip(1 << int(round(np.log2(ratio))), lo, hi))


class CullPlan(NamedTuple):
    order: object          # (N,) facet permutation (stable along-track sort):
    #                        int64 ndarray, or an int64 device tensor when
    #                        the plan was made for a CUDA device
    block_size: int
    n_blocks: int
    off: np.ndarray        # (T,) int32 first block of each trace window
    n_win: int             # blocks per window


def cull_plan(positions, centers, *, t0, dt, n_samples, c, block_size,
              target_pairs, window_cull=True, device=None):
    """Order + windows as coherent.py:284-296 / multilayer.py:684-697.

    With a CUDA ``device`` the sort and the window searches run there: the
    projections are computed on the host exactly as the reference computes
    them, uploaded, stably sorted (equal keys keep their index order, -0.0
    counts as +0.0, as in NumPy's comparison) and searched on the device;
    the permutation stays there as an int64 tensor and only the per-trace
    window offsets come back."""
    pos = np.asarray(positions, np.float64)
    cen = np.asarray(centers, np.float64)
    n = len(cen)
    bs = min(block_size or auto_block_size(len(pos), target_pairs), n)
    n_blocks = -(-n // bs)
    d = pos[-1, :2] - pos[0, :2]
    nrm = np.linalg.norm(d)
    axis = d / nrm if nrm > 0 else np.array([1.0, 0.0])
    s_f = cen[:, :2] @ axis
    if device is not None and torch.device(device).type == "cuda":
        return _cull_plan_device(s_f + 0.0, pos[:, :2] @ axis, bs, n_blocks,
                                 t0, dt, n_samples, c, window_cull, device)
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


def _cull_plan_device(s_f, s_t, bs, n_blocks, t0, dt, n_samples, c,
                      window_cull, device):
    keys = torch.from_numpy(s_f).to(device)
    s_sorted, order = torch.sort(keys, stable=True)
    if not window_cull:
        return CullPlan(order, bs, n_blocks, np.zeros(len(s_t), np.int32),
                        int(n_blocks))
    reach = window_reach_m(t0, dt, n_samples, c)
    lo_v = torch.from_numpy(s_t - reach).to(device)
    hi_v = torch.from_numpy(s_t + reach).to(device)
    lo = torch.searchsorted(s_sorted, lo_v, right=False)
    hi = torch.searchsorted(s_sorted, hi_v, right=True)
    lh = torch.stack([lo, hi]).cpu().numpy()
    b_lo = lh[0] // bs
    b_hi = np.minimum(-(-lh[1] // bs), n_blocks)
    n_win = int(max(1, int((b_hi - b_lo).max())))
    off = np.minimum(b_lo, n_blocks - n_win).astype(np.int32)
    return CullPlan(order, bs, n_blocks, off, n_win)


def group_within_blocks(plan, key):
    """The plan with its facet order regrouped inside every culling block by
    ``key`` (per facet, in the caller's facet order): facets of similar key
    become warp neighbours. Used with per-facet roughness, whose series
    length grows with the rms height: lanes of a warp then run similar
    trip counts. Block membership -- and so every trace's window -- is
    unchanged; only the summation order inside a block moves."""
    order, bs = plan.order, plan.block_size
    if isinstance(order, torch.Tensor):
        k = torch.as_tensor(np.ascontiguousarray(key, np.float64),
                            device=order.device).index_select(0, order)
        by_key = torch.sort(k, stable=True)[1]
        blk = torch.div(by_key, bs, rounding_mode="floor")
        by_blk = torch.sort(blk, stable=True)[1]
        return plan._replace(order=order.index_select(0,
                                                      by_key[by_blk]))
    k = np.asarray(key, np.float64)[order]
    perm = np.lexsort((k, np.arange(len(order)) // bs))
    return plan._replace(order=order[perm])
