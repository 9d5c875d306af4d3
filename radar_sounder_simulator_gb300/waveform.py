"""Pulse compression of kernel output on the GPU (soundersim ``waveform.py``).

Same functions and argument meaning as the reference module:

* ``compressed_pulse(bandwidth, pulse_length, dt, window, construction)``
  (waveform.py:79-123) builds the sampled, peak-normalised compressed pulse
  on the host -- the analytic raised-cosine windowed sinc or the explicit
  LFM matched filter decimated onto the dt lattice;
* ``convolve_fast_time(arr, kernel, center)`` (waveform.py:126-138) is the
  'same'-mode fast-time convolution, run by ``ss_range_compress_plan`` /
  ``ss_range_compress_apply`` (FFT, the reference's method, in float64 or
  in double-float on the FP32 pipe) or, beyond 8192 points,
  ``ss_range_compress`` (compensated direct sum);
* ``apply_waveform(out, radar, mode)`` (waveform.py:141-160) applies the
  configured waveform: identity for ``kind="delta"``, complex convolution
  in coherent mode, |p|^2 power-envelope convolution in incoherent mode
  only when ``incoherent_envelope`` is set.

``compress_tensor`` is the device-resident form for callers that keep the
kernel output on the GPU; ``RangeCompressor`` transforms a pulse once for
many arrays.
"""

import ctypes as C
import warnings

import numpy as np
import torch

from . import _lib

_WINDOW_A = {"none": 1.0, "hann": 0.5, "hamming": 0.54}


def compressed_pulse(bandwidth, pulse_length, dt, window="hann",
                     construction="analytic"):
    """Sampled compressed pulse p(m dt), m in [-M, M]; returns ``(p, M)``
    with ``p[M] = 1`` (waveform.py:79-101 analytic, :104-123 chirp)."""
    if construction == "chirp":
        return _chirp_pulse(bandwidth, pulse_length, dt, window)
    a = _WINDOW_A[window]
    if bandwidth * pulse_length < 10.0:
        warnings.warn(
            f"chirp time-bandwidth product {bandwidth * pulse_length:.1f} < "
            "10: the stationary-phase compressed-pulse model is inaccurate "
            "for such short pulses")
    m = int(np.ceil(pulse_length / dt))
    x = bandwidth * dt * np.arange(-m, m + 1)
    # raised-cosine window in frequency = three shifted sincs in time
    p = (a * np.sinc(x) + 0.5 * (1.0 - a) * (np.sinc(x - 1.0) +
                                             np.sinc(x + 1.0))) / a
    return p, m


def _chirp_pulse(bandwidth, pulse_length, dt, window):
    """Matched-filter output of a windowed LFM chirp sampled at >= 2B and
    decimated onto the dt lattice (waveform.py:104-123)."""
    a = _WINDOW_A[window]
    m = int(np.ceil(pulse_length / dt))
    over = max(1, int(np.ceil(2.0 * bandwidth * dt)))
    dts = dt / over
    n = int(np.ceil(pulse_length / dts)) | 1
    t = (np.arange(n) - (n - 1) / 2) * dts
    s = np.exp(1j * np.pi * (bandwidth / pulse_length) * t * t)
    w = a + (1.0 - a) * np.cos(2.0 * np.pi * t / pulse_length)
    ref = np.conj(s[::-1]) * w
    nfft = 1 << (2 * n - 2).bit_length()
    y = np.fft.ifft(np.fft.fft(s, nfft) * np.fft.fft(ref, nfft))[:2 * n - 1]
    y = y / y[n - 1]
    p = np.zeros(2 * m + 1, np.complex128)
    j = np.arange(-m, m + 1)
    idx = n - 1 + j * over
    ok = (idx >= 0) & (idx < len(y)) & (np.abs(j * dt) <= pulse_length)
    p[ok] = y[idx[ok]]
    p[m] = 1.0
    return p, m


def _stage(x, power):
    """(re/im-paired or real) contiguous float view of ``x`` and its
    (T, B[, L]) shape."""
    if not x.is_cuda:
        raise ValueError("compress_tensor needs a CUDA tensor")
    xr = x
    if not power:
        if xr.is_complex():
            xr = torch.view_as_real(xr.contiguous())
        if xr.shape[-1] != 2:
            raise ValueError("complex input needs a trailing re/im axis")
        shape = xr.shape[:-1]
    else:
        if xr.is_complex():
            raise ValueError("power envelope input must be real")
        shape = xr.shape
    if len(shape) not in (2, 3):
        raise ValueError("input must be (T, B) or (T, B, L)")
    if xr.dtype not in (torch.float32, torch.float64):
        xr = xr.to(torch.float64)
    return xr.contiguous(), tuple(shape)


def _taps(kernel, power, device):
    k = np.asarray(kernel)
    if power:
        return torch.as_tensor(np.ascontiguousarray(k.real, np.float64),
                               device=device)
    kc = np.asarray(k, np.complex128)
    return torch.as_tensor(
        np.ascontiguousarray(np.stack([kc.real, kc.imag], -1)), device=device)


class RangeCompressor:
    """A compressed pulse prepared for repeated 'same'-mode fast-time
    convolutions of (T, ``n_samples``[, L]) arrays on the GPU -- the FFT
    method of ``convolve_fast_time`` (waveform.py:126-138) with its pulse
    transformed once: the constructor writes the twiddles and the pulse
    spectrum (``ss_range_compress_plan``), each ``run`` is one launch
    (``ss_range_compress_apply``, one CTA per row).

    ``precision``: "fp64" (float64 transforms, the reference's arithmetic)
    or "split" (double-float transforms on the FP32 pipe: ~1e-14 of each
    row's magnitude from the float64 ones, below the float32 rounding of
    the complex64 result). ``n_samples + len(kernel) - 1`` must be at most
    8192 (``compress_tensor(method="direct")`` takes any size).
    """

    def __init__(self, kernel, center, n_samples, *, power=False,
                 precision="fp64", device=None):
        if precision not in _lib.PREC:
            raise ValueError(f"unknown precision {precision!r}")
        self.n_taps = len(np.asarray(kernel))
        self.center, self.n_samples = int(center), int(n_samples)
        self.power, self.precision = bool(power), precision
        self._prec = _lib.PREC[precision]
        if self.n_taps <= 0 or not 0 <= self.center < self.n_taps or \
                self.n_samples <= 0:
            raise ValueError("need n_samples > 0 and 0 <= center < "
                             "len(kernel)")
        o = self._opts(1, 1, False)
        L_ = _lib.lib()
        nb = L_.ss_range_compress_plan_bytes(C.byref(o), self._prec)
        if nb == 0:
            raise ValueError("B + len(kernel) - 1 above 8192: use the "
                             "direct sum")
        # arguments checked: only now the device
        self.device = _device(device)
        self._taps = _taps(kernel, self.power, self.device)
        self.plan = torch.empty(nb, dtype=torch.uint8, device=self.device)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _lib.check(L_.ss_range_compress_plan(
            C.byref(o), self._prec, C.c_void_p(self._taps.data_ptr()),
            C.c_void_p(self.plan.data_ptr()), nb, C.c_void_p(stream)),
            "ss_range_compress_plan")

    def _opts(self, T, L, in_f64):
        return _lib.WaveformOpts(T, self.n_samples, L, self.n_taps,
                                 self.center, int(self.power), int(in_f64))

    def run(self, x, out=None):
        """Convolve ``x`` (CUDA, (T, B[, L]); complex64/complex128 or float
        re/im pairs, real with ``power``) on the current stream; returns
        complex64 (float32 clipped at 0 with ``power``)."""
        xr, shape = _stage(x, self.power)
        T, B = shape[0], shape[1]
        L = shape[2] if len(shape) == 3 else 1
        if B != self.n_samples:
            raise ValueError(f"{B} samples per trace, the plan has "
                             f"{self.n_samples}")
        if out is None:
            out = torch.empty(shape + (() if self.power else (2,)),
                              dtype=torch.float32, device=x.device)
        o = self._opts(T, L, xr.dtype == torch.float64)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _lib.check(_lib.lib().ss_range_compress_apply(
            C.byref(o), self._prec, C.c_void_p(self.plan.data_ptr()),
            self.plan.numel(), C.c_void_p(xr.data_ptr()),
            C.c_void_p(out.data_ptr()), C.c_void_p(stream)),
            "ss_range_compress_apply")
        return out if self.power else torch.view_as_complex(out)


def compress_tensor(x, kernel, center, *, power=False, out=None,
                    method="auto", precision="fp64"):
    """Device form: 'same'-mode convolution of ``x`` along dim 1.

    ``x``: CUDA tensor (T, B[, L]) -- complex64/complex128, or float
    (T, B[, L], 2) re/im pairs; with ``power`` a real (T, B[, L]) float
    tensor. ``kernel``: 1-D taps (host array or tensor), zero lag at
    ``center``. Returns complex64 (T, B[, L]) (float32 when ``power``),
    launched on the current stream. ``method``: "fft" (FFT in shared
    memory, the reference's method, in ``precision`` "fp64" or "split" as
    ``RangeCompressor``; B + len(kernel) - 1 <= 8192), "direct"
    (compensated direct sum, any size) or "auto" (FFT when it fits). A
    pulse applied to many arrays is cheaper through one ``RangeCompressor``.
    """
    if method not in ("auto", "fft", "direct"):
        raise ValueError(f"unknown method {method!r}")
    xr, shape = _stage(x, power)
    T, B = shape[0], shape[1]
    L = shape[2] if len(shape) == 3 else 1
    n_taps = len(np.asarray(kernel))
    o = _lib.WaveformOpts(T, B, L, n_taps, int(center), int(bool(power)),
                          int(xr.dtype == torch.float64))
    L_ = _lib.lib()
    fits = L_.ss_range_compress_plan_bytes(C.byref(o), 0) > 0
    if method == "fft" and not fits:
        raise ValueError("B + len(kernel) - 1 above 8192: use the direct sum")
    if method != "direct" and fits:
        if not 0 <= int(center) < n_taps:
            raise ValueError("need 0 <= center < len(kernel)")
        rc = RangeCompressor(kernel, center, B, power=power,
                             precision=precision, device=x.device)
        return rc.run(xr, out=out)
    taps = _taps(kernel, power, x.device)
    if out is None:
        out = torch.empty(shape + (() if power else (2,)),
                          dtype=torch.float32, device=x.device)
    stream = torch.cuda.current_stream(x.device).cuda_stream
    st = L_.ss_range_compress(C.byref(o), C.c_void_p(taps.data_ptr()),
                              C.c_void_p(xr.data_ptr()),
                              C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    _lib.check(st, "ss_range_compress")
    return out if power else torch.view_as_complex(out)


def _device(device):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda", torch.cuda.current_device())


def convolve_fast_time(arr, kernel, center, *, device=None,
                       precision="fp64"):
    """'Same'-mode convolution along axis 1 with the kernel's zero lag at
    ``center`` (waveform.py:126-138). ``arr`` is (traces, n_samples, ...)
    complex or real; returns complex128 of the same shape (computed on the
    GPU from the float32-rounded input, as the reference convolves the
    kernels' complex64 output). ``precision`` of the FFT transforms: "fp64"
    or "split" (``RangeCompressor``)."""
    a = np.asarray(arr)
    dev = _device(device)
    shape = a.shape
    x = a.reshape(shape[0], shape[1], -1)
    xt = torch.as_tensor(np.ascontiguousarray(
        np.stack([x.real, x.imag], -1).astype(np.float32)), device=dev)
    y = compress_tensor(xt, kernel, center, precision=precision)
    return y.cpu().numpy().astype(np.complex128).reshape(shape)


def apply_waveform(out, radar, mode, *, device=None, precision="fp64"):
    """Apply ``radar.waveform`` to a kernel output (waveform.py:141-160).

    Coherent: complex convolution with the compressed pulse, complex64
    result. Incoherent: |p|^2 power-envelope convolution, clipped at zero,
    float32 -- only when ``incoherent_envelope`` is set, else ``out`` is
    returned unchanged. ``kind="delta"`` returns ``out`` unchanged.
    ``precision`` of the FFT transforms: "fp64" or "split"
    (``RangeCompressor``).
    """
    wf = radar.waveform
    if wf.kind == "delta":
        return out
    p, m = compressed_pulse(wf.bandwidth, wf.pulse_length, radar.dt,
                            wf.window, wf.construction)
    if mode != "coherent" and not wf.incoherent_envelope:
        return out
    dev = _device(device)
    a = np.asarray(out)
    shape = a.shape
    if mode == "coherent":
        x = a.reshape(shape[0], shape[1], -1).astype(np.complex64)
        xt = torch.as_tensor(np.ascontiguousarray(x), device=dev)
        y = compress_tensor(xt, p, m, precision=precision)
        return y.cpu().numpy().reshape(shape)
    x = a.reshape(shape[0], shape[1], -1).astype(np.float32)
    xt = torch.as_tensor(np.ascontiguousarray(x), device=dev)
    y = compress_tensor(xt, np.abs(p) ** 2, m, power=True,
                        precision=precision)
    return y.cpu().numpy().reshape(shape)
