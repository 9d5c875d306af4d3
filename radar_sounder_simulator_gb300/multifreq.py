"""Frequency-sampled facet synthesis ("Mode F") on GB300.

Mirrors soundersim ``compare/multifreq.py``: ``band_frequencies`` (:45-49),
``window_weights`` (:52-55) and ``multifreq_profile`` (:58-98) with the same
arguments, alias guard and return value, plus ``multifreq_traces`` /
``prepare_multifreq``, which run the same synthesis for every trace of a
track:

    H[t, k] = sum_n contrib_n(t, f_k)
    y[t, b] = sum_k Wbar_k H[t, k] exp(2j pi (f_k - f0) twtt_b)

``contrib`` is the LPA facet field of ``kernels/coherent.py:107-128`` at
wavenumber 2 pi f_k / c (``freeze_amplitudes=False``) or with its amplitude
frozen at f0 and the exact per-frequency phase (``True``). The band
response runs in ``ss_multifreq_response`` and the synthesis in
``ss_multifreq_synth``; there is no CPU path. Extensions (keyword-only):
``precision`` ("fp64" default, or "split"), ``taper_s``, per-facet
``gamma``, and ``roughness`` (frozen amplitudes, split form; the reference
tuple as in ``coherent_cluttergram``) for multi-band rough scenes.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .coherent import _dev, rough_struct, stage_facets
from .geometry import cull_plan

_WINDOW_A = {"none": 1.0, "hann": 0.5, "hamming": 0.54}


def band_frequencies(f0, bandwidth, n_freq):
    """Midpoint samples of [f0 - B/2, f0 + B/2] (multifreq.py:45-49)."""
    return f0 - bandwidth / 2.0 + (np.arange(n_freq) + 0.5) * (bandwidth /
                                                               n_freq)


def window_weights(freqs, f0, bandwidth, window):
    """Raised-cosine compression weights W(f) (multifreq.py:52-55)."""
    a = _WINDOW_A[window]
    return a + (1.0 - a) * np.cos(2.0 * np.pi * (freqs - f0) / bandwidth)


class MultifreqPlan:
    """Device-resident inputs of one multi-frequency synthesis."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def kernel_launches(self):
        """Library kernels one ``run()`` launches: band response, chunk
        reduce, synthesis."""
        return 3

    def response(self, out=None):
        """Band response H (T, K, 2) float64 re/im on the current stream."""
        L = _lib.lib()
        nbytes = L.ss_multifreq_scratch_bytes(C.byref(self.opts), self.T,
                                              self.N)
        if nbytes == 0:
            raise ValueError("unsupported sizes for the multifreq kernel")
        if self.scratch is None or self.scratch.numel() < nbytes:
            self.scratch = torch.empty(nbytes, dtype=torch.uint8,
                                       device=self.device)
        H = out if out is not None else torch.empty(
            (self.T, self.K, 2), dtype=torch.float64, device=self.device)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = L.ss_multifreq_response(
            C.byref(self.opts), C.byref(self.fst), C.byref(self.tr),
            C.byref(self.rst), C.c_void_p(H.data_ptr()),
            C.c_void_p(self.scratch.data_ptr()), nbytes, C.c_void_p(stream))
        _lib.check(st, "ss_multifreq_response")
        return H

    def synth(self, H, out=None):
        """Compressed profiles y (T, B, 2) float64 re/im from H."""
        y = out if out is not None else torch.empty(
            (self.T, self.B, 2), dtype=torch.float64, device=self.device)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = _lib.lib().ss_multifreq_synth(
            C.byref(self.opts), self.T, C.c_void_p(H.data_ptr()),
            C.c_void_p(self.wbar.data_ptr()),
            C.c_void_p(self.twtt.data_ptr()), self.B,
            C.c_void_p(y.data_ptr()), C.c_void_p(stream))
        _lib.check(st, "ss_multifreq_synth")
        return y

    def run(self):
        return self.synth(self.response())

    def to_numpy(self, y):
        f = y.cpu().numpy()
        return f[..., 0] + 1j * f[..., 1]


def _delay_span(pos, centers, twtt, c, device):
    """max(twtt U tau) - min(twtt U tau) over all (trace, facet) pairs, the
    referee's alias measure (multifreq.py:69-76), evaluated on the device in
    trace chunks."""
    cen = torch.as_tensor(np.asarray(centers, np.float64), device=device)
    p = torch.as_tensor(np.asarray(pos, np.float64), device=device)
    lo, hi = float(np.min(twtt)), float(np.max(twtt))
    step = max(1, (1 << 26) // max(len(cen), 1))
    for s in range(0, len(p), step):
        r = torch.cdist(p[s:s + step], cen)
        lo = min(lo, 2.0 * float(r.min()) / c)
        hi = max(hi, 2.0 * float(r.max()) / c)
    return hi - lo


def prepare_multifreq(positions, centers, normals, areas, e1, e2, *, gamma,
                      f0, bandwidth, c, twtt, window="hann", n_freq=128,
                      freeze_amplitudes=False, taper_s=None, roughness=None,
                      d_phi_area=False, block_size=None, window_cull=False,
                      check_alias=True, precision="fp64", device=None):
    """Upload facets and tracks for ``multifreq_traces`` (one copy)."""
    device = torch.device(device or "cuda")
    pos = np.asarray(positions, np.float64).reshape(-1, 3)
    tw = np.asarray(twtt, np.float64).ravel()
    T, B = len(pos), len(tw)
    n = np.asarray(centers).shape[0]
    # option errors come before any device work
    if precision not in _lib.PREC:
        raise ValueError(f"unknown precision {precision!r}")
    if roughness is not None and not freeze_amplitudes:
        raise ValueError("roughness needs freeze_amplitudes=True")
    gamma_arr = np.asarray(gamma, np.float32)
    gamma_facet = gamma_arr.ndim > 0
    if gamma_facet and gamma_arr.shape != (n,):
        raise ValueError(f"per-facet gamma shape {gamma_arr.shape} != ({n},)")
    rst, s_arr, l_arr, phasors = rough_struct(roughness, d_phi_area)
    if check_alias:
        span = _delay_span(pos, centers, tw, c, device)
        if span > n_freq / bandwidth:
            raise ValueError(
                f"multifreq referee would alias: delay span {span * 1e6:.2f} "
                f"us > K/B = {n_freq / bandwidth * 1e6:.2f} us; raise n_freq "
                "or shrink the scene/window")
    dt = (tw[-1] - tw[0]) / max(B - 1, 1) if B > 1 else 1e-9
    plan = cull_plan(pos, centers, t0=tw[0], dt=dt, n_samples=B, c=c,
                     block_size=block_size, target_pairs=1 << 19,
                     window_cull=window_cull)
    fac = stage_facets(centers, normals, areas, e1, e2, plan.order, device,
                       gamma=gamma_arr if gamma_facet else None,
                       sigma=s_arr, corr=l_arr, phasors=phasors)
    pos_t = _dev(pos, np.float64, device)
    off_t = _dev(plan.off, np.int32, device)
    tr = _lib.Traces(pos_t.data_ptr(), None, None, off_t.data_ptr(), T, 0)
    freqs = band_frequencies(f0, bandwidth, n_freq)
    w = window_weights(freqs, f0, bandwidth, window)
    wbar = _dev(w / w.sum(), np.float64, device)
    tw_t = _dev(tw, np.float64, device)
    opts = _lib.MultifreqOpts(
        float(f0), float(bandwidth), float(c),
        0.0 if gamma_facet else float(gamma), float(taper_s or 0.0),
        int(n_freq), int(bool(freeze_amplitudes)), int(taper_s is not None),
        plan.block_size, plan.n_win, _lib.PREC[precision])
    return MultifreqPlan(
        opts=opts, fst=fac.struct(), tr=tr, rst=rst,
        keep=[fac, pos_t, off_t], wbar=wbar, twtt=tw_t, T=T, N=n, K=n_freq,
        B=B, device=device, precision=precision, scratch=None, cull=plan)


def multifreq_traces(positions, centers, normals, areas, e1, e2, *, gamma,
                     f0, bandwidth, c, twtt, window="hann", n_freq=128,
                     freeze_amplitudes=False, taper_s=None, roughness=None,
                     d_phi_area=False, block_size=None, window_cull=False,
                     check_alias=True, precision="fp64", device=None):
    """Compressed profiles y(twtt) (complex128, (T, B)) for every platform
    position: the per-position referee run for a whole track."""
    plan = prepare_multifreq(
        positions, centers, normals, areas, e1, e2, gamma=gamma, f0=f0,
        bandwidth=bandwidth, c=c, twtt=twtt, window=window, n_freq=n_freq,
        freeze_amplitudes=freeze_amplitudes, taper_s=taper_s,
        roughness=roughness, d_phi_area=d_phi_area, block_size=block_size,
        window_cull=window_cull, check_alias=check_alias,
        precision=precision, device=device)
    return plan.to_numpy(plan.run())


def multifreq_profile(position, centers, normals, areas, e1, e2, *, gamma,
                      f0, bandwidth, c, twtt, window="hann", n_freq=128,
                      freeze_amplitudes=False, precision="fp64",
                      device=None):
    """Compressed range profile y(twtt) (complex128) for one platform
    position (multifreq.py:58-98); raises when the K-point band sampling
    would alias (span > K/B)."""
    y = multifreq_traces(
        np.asarray(position, np.float64).reshape(1, 3), centers, normals,
        areas, e1, e2, gamma=gamma, f0=f0, bandwidth=bandwidth, c=c,
        twtt=twtt, window=window, n_freq=n_freq,
        freeze_amplitudes=freeze_amplitudes, precision=precision,
        device=device)
    return y[0]
