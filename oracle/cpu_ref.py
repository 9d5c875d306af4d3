"""Multi-core float64 host restatement of the coherent facet path (test
infrastructure and the timed CPU baseline; never on the product path).

``cpu_ref.cpp`` restates the per-pair formulas of the NumPy oracle in this
directory (smooth LPA surface pair, sequential and joint refracted pairs,
Fresnel, spreading, attenuation, fast-time bin) in C++17 with OpenMP over
traces. This module keeps the oracle's host preparation -- culling order and
windows (``geometry.culling_plan``), float32 quantisation of the facet
columns, lookup grids and affine fits (``refracted.grid_consts``), joint
padding (``refracted.joint_consts``) -- and hands the arrays to the C++
library. The reference is soundersim ``kernels/coherent.py:247-362`` and
``kernels/multilayer.py:594-770``; only the features of the multilayer
benchmark are restated (isotropic antenna, smooth facets, per-facet or
scalar gamma); other options raise ``NotImplementedError``.

    build()                      # g++ -O3 -fopenmp -ffp-contract=off
    coherent_cluttergram(...)    # oracle.lpa signature subset
    refracted_cluttergram(...)   # oracle.refracted signature subset
"""

import ctypes as C
import os
import subprocess

import numpy as np

from .geometry import culling_plan
from .refracted import grid_consts, joint_consts

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_ref.cpp")
LIB = os.path.join(HERE, "_build", "libcpuref.so")
_lib = None


def build(force=False):
    """Compile the restatement (seconds); returns the library path."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB + ".tmp"
    cmd = [cxx, "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off",
           "-fPIC", "-shared", SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cpu_ref build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        d, i64, i, f = (C.POINTER(C.c_double), C.POINTER(C.c_int64),
                        C.c_int, C.c_double)
        L.cpu_ref_coherent.restype = C.c_int
        L.cpu_ref_coherent.argtypes = [i, d, i64, i64, d, d, d, d, d, d, f,
                                       f, f, f, f, i, d, d]
        fpp = C.POINTER(C.POINTER(C.c_float))
        ip = C.POINTER(C.c_int)
        L.cpu_ref_refracted.restype = C.c_int
        L.cpu_ref_refracted.argtypes = [i, d, i64, i64, d, d, d, d, d, d, f,
                                        i, i, fpp, fpp, ip, ip, d, d, d, d,
                                        d, d, i, i, i, i, f, f, f, f, i, d,
                                        d]
        L.cpu_ref_threads.restype = C.c_int
        L.cpu_ref_threads.argtypes = []
        L.cpu_ref_set_threads.restype = None
        L.cpu_ref_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def threads():
    """OpenMP threads the library runs with (OMP_NUM_THREADS or all)."""
    return int(lib().cpu_ref_threads())


def set_threads(n):
    """Run the following calls on ``n`` OpenMP threads."""
    lib().cpu_ref_set_threads(int(n))


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def _windows(plan, n):
    order, bs, _, off, n_win = plan
    lo = np.asarray(off, np.int64) * bs
    hi = np.minimum((np.asarray(off, np.int64) + n_win) * bs, n)
    return order, np.ascontiguousarray(lo), np.ascontiguousarray(hi)


def _facets(order, *cols):
    return [np.ascontiguousarray(np.asarray(a, np.float32)[order],
                                 np.float64) for a in cols]


def coherent_cluttergram(positions, u_ct, centers, normals, areas, e1, e2, *,
                         k, gamma, t0, dt, n_samples, c, block_size=None,
                         window_cull=True, **unsupported):
    """Smooth isotropic surface sum, float64 (oracle.lpa conventions).
    Returns (field complex128 (T, n), dropped float64 (T,))."""
    if any(v not in (None, False) for v in unsupported.values()):
        raise NotImplementedError(
            f"not restated in C++: {sorted(unsupported)}")
    pos = np.ascontiguousarray(positions, np.float64)
    n = len(centers)
    plan = culling_plan(pos, centers, t0=t0, dt=dt, n_samples=n_samples,
                        c=c, block_size=block_size, target_pairs=1 << 19,
                        window_cull=window_cull)
    order, lo, hi = _windows(plan, n)
    cf, nf, af, f1, f2 = _facets(order, centers, normals, areas, e1, e2)
    g = np.asarray(gamma)
    gf = (np.ascontiguousarray(np.asarray(g, np.float32)[order], np.float64)
          if g.ndim else None)
    T = len(pos)
    field = np.zeros((T, n_samples, 2))
    drop = np.zeros(T)
    st = lib().cpu_ref_coherent(
        T, _p(pos), _p(lo, C.c_int64), _p(hi, C.c_int64), _p(cf), _p(nf),
        _p(af), _p(f1), _p(f2), _p(gf) if gf is not None else None,
        float(gamma) if gf is None else 0.0, float(k), float(t0), float(dt),
        float(c), int(n_samples), _p(field), _p(drop))
    if st:
        raise RuntimeError(f"cpu_ref_coherent failed ({st})")
    return field[..., 0] + 1j * field[..., 1], drop


def refracted_cluttergram(positions, u_ct, target, crossed, eps_leg,
                          att_leg, *, mode, t0, dt, n_samples, c, gamma=0.0,
                          k0=None, refraction="sequential", pad_to=None,
                          joint_newton=6, joint_backtrack=4, block_size=None,
                          window_cull=True, **unsupported):
    """Coherent refracted target sum, float64 (oracle.refracted
    conventions). Returns (field complex128 (T, n), dropped float64 (T,))."""
    if mode != "coherent":
        raise NotImplementedError("only coherent mode is restated in C++")
    if any(v not in (None, False) for v in unsupported.values()):
        raise NotImplementedError(
            f"not restated in C++: {sorted(unsupported)}")
    joint = refraction == "joint"
    pos = np.ascontiguousarray(positions, np.float64)
    eps = np.asarray(eps_leg, np.float64)
    n_leg = np.sqrt(eps)
    att = np.asarray(att_leg, np.float64)
    grids = []
    if joint:
        gc, gn, coef, shp, mp, mn, kp = joint_consts(
            crossed, pad_to or len(crossed), pos[:, 2].min())
        n_leg = np.concatenate([np.full(kp, n_leg[0]), n_leg])
        eps = np.concatenate([np.full(kp, eps[0]), eps])
        att = np.concatenate([np.full(kp, att[0]), att])
        for i in range(len(mp)):
            ny, nx = int(shp[i][0]), int(shp[i][1])
            grids.append((np.ascontiguousarray(gc[i, :ny, :nx]),
                          np.ascontiguousarray(gn[i, :ny, :nx]), coef[i],
                          mp[i], mn[i]))
    else:
        kp = 0
        for f in crossed:
            g_c, g_n, coef, mp, mn = grid_consts(f)
            grids.append((np.ascontiguousarray(g_c), np.ascontiguousarray(g_n),
                          coef, mp, mn))
    ni = len(grids)
    n = len(target.centers)
    plan = culling_plan(pos, target.centers, t0=t0, dt=dt,
                        n_samples=n_samples, c=c,
                        block_size=block_size or (4096 if joint else None),
                        target_pairs=1 << 18, window_cull=window_cull)
    order, lo, hi = _windows(plan, n)
    cf, nf, af, f1, f2 = _facets(order, target.centers, target.normals,
                                 target.areas, target.e1, target.e2)
    g = np.asarray(gamma, np.float64)
    gf = np.ascontiguousarray(g[order]) if g.ndim else None
    FP = C.POINTER(C.c_float)
    gcs = (FP * ni)(*[_p(t[0], C.c_float) for t in grids])
    gns = (FP * ni)(*[_p(t[1], C.c_float) for t in grids])
    ny = np.ascontiguousarray([t[0].shape[0] for t in grids], np.int32)
    nx = np.ascontiguousarray([t[0].shape[1] for t in grids], np.int32)
    coef = np.ascontiguousarray(np.stack([np.asarray(t[2], np.float64)
                                          .reshape(6) for t in grids]))
    mp = np.ascontiguousarray(np.stack([t[3] for t in grids]), np.float64)
    mn = np.ascontiguousarray(np.stack([t[4] for t in grids]), np.float64)
    legs = [np.ascontiguousarray(v, np.float64) for v in (n_leg, eps, att)]
    T = len(pos)
    field = np.zeros((T, n_samples, 2))
    drop = np.zeros(T)
    st = lib().cpu_ref_refracted(
        T, _p(pos), _p(lo, C.c_int64), _p(hi, C.c_int64), _p(cf), _p(nf),
        _p(af), _p(f1), _p(f2), _p(gf) if gf is not None else None,
        0.0 if gf is not None else float(g), ni, int(kp), gcs, gns,
        _p(ny, C.c_int), _p(nx, C.c_int), _p(coef), _p(mp), _p(mn),
        _p(legs[0]), _p(legs[1]), _p(legs[2]), len(legs[0]), int(joint),
        int(joint_newton),
        int(joint_backtrack), 0.0 if k0 is None else float(k0), float(t0),
        float(dt), float(c), int(n_samples), _p(field), _p(drop))
    if st:
        raise RuntimeError(f"cpu_ref_refracted failed ({st})")
    return field[..., 0] + 1j * field[..., 1], drop
