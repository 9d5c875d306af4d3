"""Float64 CPU oracle for the coherent / refracted facet kernels.

TEST INFRASTRUCTURE, NOT PRODUCT CODE. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import anything under ``oracle/``, and only as the checker (or the timed
CPU baseline) -- never as the thing measured or shipped. The product path
(``radar_sounder_simulator_gb300``) never imports it and fails loudly when
its CUDA library is missing.

Contents: a NumPy float64 restatement of the reference simulator's hot path
(soundersim, paths relative to ``src/soundersim/``), each function citing the
reference file:line it follows:

- ``geometry``  -- binning and along-track window culling (kernels/geometry.py)
- ``roughness`` -- Gerekos 2023 D_Phi series, Faddeeva, attenuation
                   (roughness.py)
- ``antenna``   -- in-kernel one-way field gains (antenna.py gain_fn)
- ``lpa``       -- surface LPA facet field + binned coherent cluttergram
                   (kernels/coherent.py)
- ``refraction``-- two-point Snell solve and joint N-interface solve
                   (refraction.py, refraction_joint.py)
- ``refracted`` -- refracted multilayer cluttergram (kernels/multilayer.py)
- ``waveform``  -- compressed pulse + fast-time convolution (waveform.py)
- ``multifreq`` -- frequency-sampled synthesis (compare/multifreq.py)

Parity is pinned: ``tests/golden/make_golden.py`` runs the unmodified
reference source (with a NumPy stand-in for JAX) and freezes its outputs in
``tests/golden/*.npz``; ``tests/test_oracle_golden.py`` checks this oracle
against them.

Precision conventions (identical to the GPU float64 form): facet geometry is
quantised to float32 first (as the reference's ``blocks()`` does), then all
arithmetic runs in float64; platform positions and the radar scalars
(k, t0, dt, c) stay float64; phases are absolute (no reference-range fold);
bins accumulate in complex128.
"""
