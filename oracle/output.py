"""Per-trace output products in float64 NumPy (oracle).

Test infrastructure only: the GPU path never imports this module.

Restates the facet scans of soundersim ``output.py:47-82``
(``build_dataset``): the nadir facet (horizontally nearest centre, first
index on ties), ``nadir_twtt`` = 2 (z_platform - z_facet) / c, and the first
return: the earliest exact float64 twtt 2r/c over facets inside
[t0, t0 + n_samples dt), first index on ties, +inf (facet 0) when no facet
is in the window. Traces are processed in blocks so memory stays bounded.
"""

import numpy as np


def trace_products(centers, positions, t0, dt, n_samples, c, block=8):
    cen = np.asarray(centers, np.float64)
    pos = np.asarray(positions, np.float64)
    T = len(pos)
    nadir_idx = np.zeros(T, np.int64)
    first_idx = np.zeros(T, np.int64)
    first_twtt = np.zeros(T)
    t_end = t0 + n_samples * dt
    for a in range(0, T, block):
        p = pos[a:a + block]
        d2 = ((cen[None, :, :2] - p[:, None, :2]) ** 2).sum(-1)
        nadir_idx[a:a + block] = d2.argmin(axis=1)
        r = np.linalg.norm(cen[None, :, :] - p[:, None, :], axis=-1)
        ft = 2.0 * r / c
        ft = np.where((ft >= t0) & (ft < t_end), ft, np.inf)
        fi = ft.argmin(axis=1)
        first_idx[a:a + block] = fi
        first_twtt[a:a + block] = ft[np.arange(len(p)), fi]
    nadir_twtt = 2.0 * (pos[:, 2] - cen[nadir_idx, 2]) / c
    return nadir_twtt, nadir_idx, first_twtt, first_idx
