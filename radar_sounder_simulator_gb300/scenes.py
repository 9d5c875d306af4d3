"""Seeded synthetic scenes for the benchmark configurations and tests.

Host-side inputs only (no kernel code). Facets follow the reference's corner
rule for rectangular DEM cells (soundersim ``scene.py:156-166``): mean edge
vectors e1 (along +column) and e2 (along +row), centroid = mean of the four
corners, area = |e1 x e2|, normal = (e1 x e2)/area oriented +z. Surfaces are
Gaussian random fields with an isotropic Gaussian (``compare/haynes.py``
generator form) or exponential correlation function, built by circular FFT
filtering of white noise and normalised by the filter's energy so the field
variance is exactly the target (no per-realisation rescaling).
"""

from types import SimpleNamespace

import numpy as np

C_LIGHT = 299792458.0


def random_field(n, dx, corr_len, rms, rng, acf="exponential"):
    """(n, n) zero-mean random field with rms ``rms`` and the given ACF."""
    kx = 2.0 * np.pi * np.fft.fftfreq(n, d=dx)
    k2 = kx[:, None] ** 2 + kx[None, :] ** 2
    if acf == "exponential":
        # 2-D spectrum of exp(-r/l): 2 pi l^2 (1 + k^2 l^2)^(-3/2)
        spec = 2.0 * np.pi * corr_len ** 2 * (1.0 + k2 * corr_len ** 2) ** -1.5
    elif acf == "gaussian":
        # 2-D spectrum of exp(-r^2/l^2): pi l^2 exp(-k^2 l^2 / 4)
        spec = np.pi * corr_len ** 2 * np.exp(-k2 * corr_len ** 2 / 4.0)
    else:
        raise ValueError(f"unknown acf {acf!r}")
    h = np.sqrt(spec)
    w = rng.standard_normal((n, n))
    z = np.real(np.fft.ifft2(np.fft.fft2(w) * h))
    return rms * z / np.sqrt(np.mean(h * h))


def facets_from_vertices(X, Y, Z):
    """Rectangular facets of a vertex grid (scene.py:156-166 corner rule).
    Returns a Facets-like namespace with ``cell`` and ``grid_shape`` for the
    refracted kernel's lookup tables."""
    V = np.stack([X, Y, Z], axis=-1)
    v00, v01 = V[:-1, :-1], V[:-1, 1:]
    v10, v11 = V[1:, :-1], V[1:, 1:]
    e1 = ((v01 + v11) - (v00 + v10)) / 2.0
    e2 = ((v10 + v11) - (v00 + v01)) / 2.0
    centers = ((v00 + v01 + v10 + v11) / 4.0).reshape(-1, 3)
    raw = np.cross(e1, e2).reshape(-1, 3)
    areas = np.linalg.norm(raw, axis=1)
    normals = raw / areas[:, None]
    normals *= np.where(normals[:, 2] < 0.0, -1.0, 1.0)[:, None]
    ny, nx = X.shape[0] - 1, X.shape[1] - 1
    ci, cj = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    return SimpleNamespace(
        centers=centers, normals=normals, areas=areas,
        e1=e1.reshape(-1, 3), e2=e2.reshape(-1, 3),
        cell=np.stack([ci.ravel(), cj.ravel()], axis=1), grid_shape=(ny, nx),
        phase_keys=None)


def surface(n_cells, spacing, rms, corr_len, z0, rng, acf="exponential"):
    """Square patch of n_cells^2 facets centred on the origin."""
    ax = (np.arange(n_cells + 1) - n_cells / 2.0) * spacing
    X, Y = np.meshgrid(ax, ax)
    Z = z0 + random_field(n_cells + 1, spacing, corr_len, rms, rng, acf)
    return facets_from_vertices(X, Y, Z)


def straight_track(n, spacing, altitude):
    """Track along +x through the origin; u_ct = (0, -1, 0) (nav.py:25-29:
    cross-track-right of +x travel in an ENU frame)."""
    x = (np.arange(n) - (n - 1) / 2.0) * spacing
    pos = np.column_stack([x, np.zeros(n), np.full(n, float(altitude))])
    uct = np.tile([0.0, -1.0, 0.0], (n, 1))
    return pos, uct


def fresnel_normal(eps1, eps2):
    """Normal-incidence field reflection (physics.py:16-21)."""
    n1, n2 = np.sqrt(eps1), np.sqrt(eps2)
    return (n1 - n2) / (n1 + n2)


def eps_kovacs(rho):
    """Kovacs density -> permittivity (firn.py:19-21)."""
    return (1.0 + 0.845 * np.asarray(rho) / 1000.0) ** 2


def firn_n_eff(depth, rho_surface=350.0, rho_ice=917.0, scale=30.0):
    """Delay-equivalent index of the firn column over ``depth`` metres:
    (1/depth) int_0^depth sqrt(eps(rho(z))) dz with rho(z) = rho_ice -
    (rho_ice - rho_surface) exp(-z/scale)."""
    z = np.linspace(0.0, depth, 20001)
    rho = rho_ice - (rho_ice - rho_surface) * np.exp(-z / scale)
    n = np.sqrt(eps_kovacs(rho))
    return float(np.trapezoid(n, z) / depth)


def window(pos, centers, *, n_samples, dt, lead_m=200.0, c=C_LIGHT):
    """t0 = 2 (min slant range - lead) / c (the configs' window rule)."""
    step = max(1, len(pos) // 256)
    r = np.linalg.norm(pos[::step, None, :] - centers[None, ::97],
                       axis=-1).min()
    return 2.0 * (r - lead_m) / c


def config1(seed=1):
    """Plain single-surface coherent run: 128^2 facets of 100 m,
    exponential ACF (1 km, 50 m rms), air/ice (eps 3.15) Fresnel, isotropic
    antenna, 256 traces at 50 m, 20 km altitude, 60 MHz, dt = 1/(2 x 15 MHz),
    2048 bins."""
    rng = np.random.default_rng(seed)
    f = surface(128, 100.0, 50.0, 1000.0, 0.0, rng)
    pos, uct = straight_track(256, 50.0, 20000.0)
    f0, bw = 60e6, 15e6
    dt = 1.0 / (2.0 * bw)
    t0 = window(pos, f.centers, n_samples=2048, dt=dt)
    kw = dict(k=2 * np.pi * f0 / C_LIGHT, gamma=fresnel_normal(1.0, 3.15),
              t0=t0, dt=dt, n_samples=2048, c=C_LIGHT)
    return SimpleNamespace(facets=f, pos=pos, uct=uct, kw=kw, f0=f0, bw=bw,
                           pulse_length=20e-6)


def config2(seed=2, n_cells=512, n_traces=1024, spacing=50.0,
            trace_spacing=25.0, line_offset_y=0.0):
    """Multilayer with refraction: surface + horizons at 300 m and 1200 m +
    bed at 2500 m, each n_cells^2 facets of ``spacing`` metres; 1024 traces
    at 20 km; 60 MHz / 15 MHz.

    Choices where the configuration is silent:
    horizon ACF exponential with 1 km correlation; bed relief exponential,
    5 km; relative permittivity contrast 1e-3 at both horizons (their target
    reflection coefficient fresnel_normal(eps, eps (1 + 1e-3))); firn column
    above the first horizon as one medium of delay-equivalent index; 25 m
    trace spacing; bed reflectivity +10^(R/20) with R ~ U[-30, -5] dB.
    ``line_offset_y`` shifts the track cross-track (one line per GPU)."""
    rng = np.random.default_rng(seed)
    surf = surface(n_cells, spacing, 20.0, 5000.0, 0.0, rng)
    h1 = surface(n_cells, spacing, 5.0, 1000.0, -300.0, rng)
    h2 = surface(n_cells, spacing, 5.0, 1000.0, -1200.0, rng)
    bed = surface(n_cells, spacing, 300.0, 5000.0, -2500.0, rng)
    pos, uct = straight_track(n_traces, trace_spacing, 20000.0)
    pos[:, 1] += line_offset_y
    n_firn = firn_n_eff(300.0)
    eps_ice = 3.15
    eps = [1.0, n_firn ** 2, eps_ice, eps_ice * (1.0 + 1e-3),
           eps_ice * (1.0 + 1e-3) ** 2]
    att = [0.0, 10.0, 10.0, 10.0, 10.0]
    f0, bw = 60e6, 15e6
    dt = 1.0 / (2.0 * bw)
    t0 = window(pos, surf.centers, n_samples=2048, dt=dt)
    r_db = rng.uniform(-30.0, -5.0, len(bed.centers))
    gammas = [fresnel_normal(eps[0], eps[1]),
              fresnel_normal(eps_ice, eps_ice * (1.0 + 1e-3)),
              fresnel_normal(eps[2], eps[3]),
              10.0 ** (r_db / 20.0)]
    return SimpleNamespace(
        layers=[surf, h1, h2, bed], names=["surface", "h1", "h2", "bed"],
        pos=pos, uct=uct, eps=eps, att=att, gammas=gammas, f0=f0, bw=bw,
        k0=2 * np.pi * f0 / C_LIGHT, t0=t0, dt=dt, n_samples=2048,
        c=C_LIGHT, refraction="joint")


def n_terms_for(x_max):
    """D_Phi series length for the largest (sigma K)^2 of a run:
    ceil(x + 6 sqrt(x) + 5) clipped to [10, 300] (roughness.py:189-196)."""
    x = float(x_max)
    return int(np.clip(np.ceil(x + 6.0 * np.sqrt(x) + 5.0), 10, 300))


def speckle_phasors(n, seed):
    """Unit-variance complex Gaussian speckle phasors, complex64, drawn the
    way the reference's ``speckle_phasors(n, seed)`` draws them
    (roughness.py:199-204: a fresh ``default_rng(seed)``, real parts then
    imaginary parts), so a keyed seed such as ``(scene_seed, layer)`` gives
    the reference's own phasors bit for bit."""
    rng = np.random.default_rng(seed)
    ph = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return (ph / np.sqrt(2.0)).astype(np.complex64)


def config3(seed=3, n_cells=512, n_traces=2048, spacing=25.0,
            bed_depth=1000.0):
    """Sub-facet roughness, multi-frequency: the config-1 statistics
    (exponential ACF 1 km, 50 m rms) over the same 12.8 km square at 25 m
    facets (512^2, inside the 450 MHz LPA facet limit at 20 km), surface and
    a bed under ``bed_depth`` m of ice; per-facet bed rms height log-normal
    (median 0.3 m, sigma_log 0.7), correlation length U[5, 50] m,
    exponential ACF (area-only D_Phi with the 0.05 taper); surface rms
    U[0.05, 0.5] m with the same correlation lengths; 2048 traces at 20 km;
    bands at 30, 60, 150 and 450 MHz of 10% bandwidth."""
    rng = np.random.default_rng(seed)
    surf = surface(n_cells, spacing, 50.0, 1000.0, 0.0, rng)
    bed = surface(n_cells, spacing, 50.0, 1000.0, -bed_depth, rng)
    n = n_cells * n_cells
    pos, uct = straight_track(n_traces, 12800.0 / n_traces, 20000.0)
    eps = [1.0, 3.15]
    rough = dict(
        surface=dict(sigma=rng.uniform(0.05, 0.5, n),
                     corr=rng.uniform(5.0, 50.0, n),
                     phasors=speckle_phasors(n, (seed, 0))),
        bed=dict(sigma=np.exp(np.log(0.3) + 0.7 * rng.standard_normal(n)),
                 corr=rng.uniform(5.0, 50.0, n),
                 phasors=speckle_phasors(n, (seed, 1))))
    bands = [30e6, 60e6, 150e6, 450e6]
    return SimpleNamespace(surface=surf, bed=bed, pos=pos, uct=uct, eps=eps,
                           att=[0.0, 10.0], rough=rough, bands=bands,
                           frac_bw=0.10, n_freq=1024, c=C_LIGHT,
                           gamma_surface=fresnel_normal(1.0, 3.15),
                           gamma_bed=fresnel_normal(3.15, 9.0))


def config3_band(cfg, f0):
    """Fast-time window and series lengths of one band of the roughness
    configuration: dt = 1/(2 B) for the 10% bandwidth, n_samples covering
    the surface and the bed under 1000 m of ice plus 3 km of slant, t0 from
    the surface's nearest range, and the reference's D_Phi series lengths
    (n_terms_for) for the largest surface rms height and the 0.999 quantile
    of the bed's (in ice). Returns a dict (f0, bw, k0, dt, n_s, t0, nt_s,
    nt_b)."""
    bw = cfg.frac_bw * f0
    dt = 1.0 / (2.0 * bw)
    k0 = 2 * np.pi * f0 / cfg.c
    n_s = int(np.ceil(2 * (1000.0 * np.sqrt(3.15) + 3000.0) / cfg.c / dt))
    t0 = window(cfg.pos, cfg.surface.centers, n_samples=n_s, dt=dt)
    rs, rb = cfg.rough["surface"], cfg.rough["bed"]
    nt_s = n_terms_for((2 * k0 * rs["sigma"].max()) ** 2)
    nt_b = n_terms_for((2 * k0 * np.sqrt(cfg.eps[1]) *
                        np.quantile(rb["sigma"], 0.999)) ** 2)
    return dict(f0=f0, bw=bw, k0=k0, dt=dt, n_s=n_s, t0=t0, nt_s=nt_s,
                nt_b=nt_b)


def gaussian_beam_table(beamwidth_deg, n=64):
    """Tabulated one-way field gain of a Gaussian beam whose two-way power
    is -3 dB at half the beamwidth: g(theta) = 2^(-(theta/theta_h)^2 / 4)
    (g^4 = 1/2 at theta_h). Returns (angles (n,), gains (n,)) over
    [0, pi/2], the ``tabulated`` pattern's (pa, pb)."""
    th = np.linspace(0.0, np.pi / 2, n)
    th_h = np.radians(beamwidth_deg) / 2.0
    return th, 2.0 ** (-((th / th_h) ** 2) / 4.0)


def config4_instance(i, n_samples=2048, facet_m=25.0):
    """One instance of the batched design sweep (seed 4000 + i): altitude
    U[12, 25] km, centre frequency log-uniform in [30, 450] MHz with 15%
    bandwidth, beamwidth U[20, 90] deg (Gaussian tabulated pattern, boresight
    nadir), U{256..4096} traces at 25 m, U{256..1024}^2 facets of 25 m with
    the config-1 statistics (exponential ACF 1 km, 50 m rms)."""
    rng = np.random.default_rng(4000 + i)
    alt = rng.uniform(12e3, 25e3)
    f0 = float(np.exp(rng.uniform(np.log(30e6), np.log(450e6))))
    bw = 0.15 * f0
    beam = rng.uniform(20.0, 90.0)
    T = int(rng.integers(256, 4097))
    ncell = int(rng.integers(256, 1025))
    f = surface(ncell, facet_m, 50.0, 1000.0, 0.0, rng)
    pos, uct = straight_track(T, 25.0, alt)
    dt = 1.0 / (2.0 * bw)
    t0 = window(pos, f.centers, n_samples=n_samples, dt=dt)
    pa, pb = gaussian_beam_table(beam)
    pv = np.tile([0.0, 0.0, -1.0], (T, 1))
    kw = dict(k=2 * np.pi * f0 / C_LIGHT, gamma=fresnel_normal(1.0, 3.15),
              t0=t0, dt=dt, n_samples=n_samples, c=C_LIGHT,
              pattern=("tabulated", pv, pa, pb))
    return SimpleNamespace(facets=f, pos=pos, uct=uct, kw=kw, f0=f0,
                           beam=beam, T=T, n_cells=ncell)


def config5(seed=5, n_cells=512, n_traces=1024, spacing=25.0,
            bed_depth=1000.0):
    """Differentiation: the config-3 scene geometry (surface over a bed under
    ``bed_depth`` m of ice, 512^2 facets of 25 m each), 1024 traces at
    20 km, 60 MHz; bed reflectivity R ~ U[-30, -5] dB, rms height
    log-normal (median 0.3 m, sigma_log 0.7), correlation length 10 m,
    attenuation 10 dB/km; the target radargram comes from R + N(0, 1 dB),
    sigma x exp(N(0, 0.1)) and alpha + 1 dB/km."""
    rng = np.random.default_rng(seed)
    surf = surface(n_cells, spacing, 50.0, 1000.0, 0.0, rng)
    bed = surface(n_cells, spacing, 50.0, 1000.0, -bed_depth, rng)
    n = n_cells * n_cells
    pos, uct = straight_track(n_traces, 12800.0 / n_traces, 20000.0)
    f0 = 60e6
    dt = 1.0 / (2.0 * 15e6)
    t0 = 2.0 * (20000.0 - 200.0) / C_LIGHT
    R = rng.uniform(-30.0, -5.0, n)
    sig = np.exp(np.log(0.3) + 0.7 * rng.standard_normal(n))
    R_hat = R + rng.standard_normal(n)
    sig_hat = sig * np.exp(0.1 * rng.standard_normal(n))
    k_ice = 2 * np.pi * f0 / C_LIGHT * np.sqrt(3.15)
    n_terms = n_terms_for((2.0 * k_ice * np.quantile(sig, 0.999)) ** 2)
    return SimpleNamespace(surface=surf, bed=bed, pos=pos, uct=uct,
                           eps=[1.0, 3.15], alpha=10.0, k0=2 * np.pi * f0 /
                           C_LIGHT, t0=t0, dt=dt, n_samples=1024, c=C_LIGHT,
                           R=R, sig=sig, R_hat=R_hat, sig_hat=sig_hat, window=(0, 1024),
                           corr=10.0, phasors=speckle_phasors(n, (seed, 1)),
                           n_terms=n_terms)


def smoke_scene():
    """Tiny coherent case for ``__graft_entry__.smoke``."""
    rng = np.random.default_rng(7)
    f = surface(24, 30.0, 2.0, 200.0, 0.0, rng)
    pos, uct = straight_track(4, 40.0, 2000.0)
    dt = 2e-8
    t0 = window(pos, f.centers, n_samples=256, dt=dt, lead_m=20.0)
    kw = dict(k=2 * np.pi / 5.0, gamma=-0.28, t0=t0, dt=dt, n_samples=256,
              c=C_LIGHT)
    return dict(pos=pos, uct=uct, centers=f.centers, normals=f.normals,
                areas=f.areas, e1=f.e1, e2=f.e2, kw=kw)
