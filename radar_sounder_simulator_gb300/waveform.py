"""Pulse compression of kernel output on the GPU (soundersim ``waveform.py``).

Same functions and argument meaning as the reference module:

* ``compressed_pulse(bandwidth, pulse_length, dt, window, construction)``
  (waveform.py:79-123) builds the sampled, peak-normalised compressed pulse
  on the host -- the analytic raised-cosine windowed sinc or the explicit
  LFM matched filter decimated onto the dt lattice;
* ``convolve_fast_time(arr, kernel, center)`` (waveform.py:126-138) is the
  'same'-mode fast-time convolution, run by ``ss_range_compress_fft``
  (float64 FFT, the reference's method) or, beyond 8192 points,
  ``ss_range_compress`` (compensated direct sum);
* ``apply_waveform(out, radar, mode)`` (waveform.py:141-160) applies the
  configured waveform: identity for ``kind="delta"``, complex convolution
  in coherent mode, |p|^2 power-envelope convolution in incoherent mode
  only when ``incoherent_envelope`` is set.

``compress_tensor`` is the device-resident form for callers that keep the
kernel output on the GPU.
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


def compress_tensor(x, kernel, center, *, power=False, out=None,
                    method="auto"):
    """Device form: 'same'-mode convolution of ``x`` along dim 1.

    ``x``: CUDA tensor (T, B[, L]) -- complex64/complex128, or float
    (T, B[, L], 2) re/im pairs; with ``power`` a real (T, B[, L]) float
    tensor. ``kernel``: 1-D taps (host array or tensor), zero lag at
    ``center``. Returns complex64 (T, B[, L]) (float32 when ``power``),
    launched on the current stream. ``method``: "fft" (float64 FFT in shared
    memory, the reference's method; B + len(kernel) - 1 <= 8192), "direct"
    (compensated direct sum, any size) or "auto" (FFT when it fits).
    """
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
    xr = xr.contiguous()
    T, B = int(shape[0]), int(shape[1])
    L = int(shape[2]) if len(shape) == 3 else 1
    k = np.asarray(kernel)
    if power:
        taps = torch.as_tensor(np.ascontiguousarray(k.real, np.float64),
                               device=x.device)
    else:
        kc = np.asarray(k, np.complex128)
        taps = torch.as_tensor(
            np.ascontiguousarray(np.stack([kc.real, kc.imag], -1)),
            device=x.device)
    if out is None:
        out = torch.empty(tuple(shape) + (() if power else (2,)),
                          dtype=torch.float32, device=x.device)
    o = _lib.WaveformOpts(T, B, L, len(k), int(center), int(bool(power)),
                          int(xr.dtype == torch.float64))
    stream = torch.cuda.current_stream(x.device).cuda_stream
    L_ = _lib.lib()
    nfft = L_.ss_range_compress_fft_scratch_bytes(C.byref(o))
    if method == "fft" and nfft == 0:
        raise ValueError("B + len(kernel) - 1 above 8192: use the direct sum")
    if method not in ("auto", "fft", "direct"):
        raise ValueError(f"unknown method {method!r}")
    if method != "direct" and nfft > 0:
        scratch = torch.empty(nfft, dtype=torch.uint8, device=x.device)
        st = L_.ss_range_compress_fft(
            C.byref(o), C.c_void_p(taps.data_ptr()),
            C.c_void_p(xr.data_ptr()), C.c_void_p(out.data_ptr()),
            C.c_void_p(scratch.data_ptr()), nfft, C.c_void_p(stream))
        _lib.check(st, "ss_range_compress_fft")
    else:
        st = L_.ss_range_compress(C.byref(o), C.c_void_p(taps.data_ptr()),
                                  C.c_void_p(xr.data_ptr()),
                                  C.c_void_p(out.data_ptr()),
                                  C.c_void_p(stream))
        _lib.check(st, "ss_range_compress")
    return out if power else torch.view_as_complex(out)


def _device(device):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda", torch.cuda.current_device())


def convolve_fast_time(arr, kernel, center, *, device=None):
    """'Same'-mode convolution along axis 1 with the kernel's zero lag at
    ``center`` (waveform.py:126-138). ``arr`` is (traces, n_samples, ...)
    complex or real; returns complex128 of the same shape (computed on the
    GPU from the float32-rounded input, as the reference convolves the
    kernels' complex64 output)."""
    a = np.asarray(arr)
    dev = _device(device)
    shape = a.shape
    x = a.reshape(shape[0], shape[1], -1)
    xt = torch.as_tensor(np.ascontiguousarray(
        np.stack([x.real, x.imag], -1).astype(np.float32)), device=dev)
    y = compress_tensor(xt, kernel, center)
    return y.cpu().numpy().astype(np.complex128).reshape(shape)


def apply_waveform(out, radar, mode, *, device=None):
    """Apply ``radar.waveform`` to a kernel output (waveform.py:141-160).

    Coherent: complex convolution with the compressed pulse, complex64
    result. Incoherent: |p|^2 power-envelope convolution, clipped at zero,
    float32 -- only when ``incoherent_envelope`` is set, else ``out`` is
    returned unchanged. ``kind="delta"`` returns ``out`` unchanged.
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
        y = compress_tensor(xt, p, m)
        return y.cpu().numpy().reshape(shape)
    x = a.reshape(shape[0], shape[1], -1).astype(np.float32)
    xt = torch.as_tensor(np.ascontiguousarray(x), device=dev)
    y = compress_tensor(xt, np.abs(p) ** 2, m, power=True)
    return y.cpu().numpy().reshape(shape)
