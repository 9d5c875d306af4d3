"""Adjoint of windowed bed power against float64 central finite
differences of the oracle.

The reference has no gradient code (and ``jax.grad`` cannot run here), so
the gradients are pinned by central differences of the float64 oracle
forward (``oracle.refracted``, the restated multilayer.py:594-770) on the
same float32-quantised facets: relative step 2^-13 (~1.2e-4) on seeded
parameter indices, agreement within 1e-4 of the largest checked gradient
of each parameter kind.
"""

import numpy as np
import pytest
import torch

from oracle import refracted as orf
from radar_sounder_simulator_gb300 import scenes
from radar_sounder_simulator_gb300.adjoint import WindowPowerModel, db_misfit

pytestmark = pytest.mark.gpu
C = 299792458.0


def _q10(x):
    """Round to 10 significant bits so x (1 +- 2^-13) is exact in float32."""
    e = np.floor(np.log2(np.abs(x)))
    return np.round(x / 2.0 ** (e - 9)) * 2.0 ** (e - 9)


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(11)
    surf = scenes.surface(20, 25.0, 2.0, 200.0, 0.0, rng)
    bed = scenes.surface(20, 25.0, 5.0, 200.0, -200.0, rng)
    pos, uct = scenes.straight_track(6, 30.0, 800.0)
    n = len(bed.centers)
    k0 = 2 * np.pi * 60e6 / C
    dt = 1.0 / 30e6
    t0 = 2 * 760.0 / C
    ph = np.exp(2j * np.pi * rng.random(n)).astype(np.complex64)
    common = dict(t0=t0, dt=dt, n_samples=256, c=C, k0=k0)
    R = rng.uniform(-30, -5, n)
    sig = _q10(np.exp(np.log(0.3) + 0.7 * rng.standard_normal(n)))
    alpha = 10.0
    return dict(surf=surf, bed=bed, pos=pos, uct=uct, ph=ph, R=R, sig=sig,
                alpha=alpha, common=common, n=n)


def oracle_power(cs, R, sig, alpha):
    out, _ = orf.refracted_cluttergram(
        cs["pos"], cs["uct"], cs["bed"], [cs["surf"]], [1.0, 3.15],
        [0.0, alpha], mode="coherent", gamma=10.0 ** (R / 20.0),
        roughness=(sig, 4.0, cs["ph"], 40, "exponential"), d_phi_area=True,
        taper_s=0.05, refraction="sequential", **cs["common"])
    return (np.abs(out) ** 2).sum(axis=1)


@pytest.mark.parametrize("forward,tol", [("fp64", 1e-4), ("split", 5e-4)])
def test_adjoint_matches_central_differences(case, forward, tol):
    """With the float64 forward the only split-precision part is the
    adjoint's per-pair recomputation: 1e-4. With the split forward, P itself
    carries ~1e-5 relative error, which enters dL/dP: 5e-4."""
    cs = case
    model = WindowPowerModel(
        cs["pos"], cs["uct"], cs["bed"], [cs["surf"]], [1.0, 3.15],
        [0.0, cs["alpha"]], window=(0, 256), alpha_legs=(1,),
        corr_length=4.0, phasors=cs["ph"], n_terms=40, precision=forward,
        **cs["common"])
    dev = model.device
    rng = np.random.default_rng(5)
    R_hat = cs["R"] + rng.standard_normal(cs["n"])
    s_hat = _q10(cs["sig"] * np.exp(0.1 * rng.standard_normal(cs["n"])))
    P_hat = torch.as_tensor(oracle_power(cs, R_hat, s_hat, cs["alpha"] + 1.0),
                            device=dev)
    R = torch.tensor(cs["R"], device=dev, requires_grad=True)
    s = torch.tensor(cs["sig"], device=dev, requires_grad=True)
    a = torch.tensor(cs["alpha"], dtype=torch.float64, device=dev,
                     requires_grad=True)
    P = model.power(R, s, a)
    # the split-form power agrees with the float64 oracle
    P64 = oracle_power(cs, cs["R"], cs["sig"], cs["alpha"])
    assert np.abs(P.detach().cpu().numpy() / P64 - 1).max() < (
        1e-9 if forward == "fp64" else 1e-4)
    L = db_misfit(P, P_hat)
    L.backward()

    def loss(Rv, sv, av):
        Pv = oracle_power(cs, Rv, sv, av)
        return float(((10 * np.log10(Pv) - 10 * np.log10(
            P_hat.cpu().numpy())) ** 2).sum())

    h = 2.0 ** -13
    idx = rng.choice(cs["n"], size=8, replace=False)
    fd_R, fd_s = [], []
    for i in idx:
        Rp, Rm = cs["R"].copy(), cs["R"].copy()
        dR = h * abs(cs["R"][i])
        Rp[i] += dR
        Rm[i] -= dR
        fd_R.append((loss(Rp, cs["sig"], cs["alpha"]) -
                     loss(Rm, cs["sig"], cs["alpha"])) / (2 * dR))
        sp, sm = cs["sig"].copy(), cs["sig"].copy()
        ds = h * cs["sig"][i]
        sp[i] += ds
        sm[i] -= ds
        fd_s.append((loss(cs["R"], sp, cs["alpha"]) -
                     loss(cs["R"], sm, cs["alpha"])) / (2 * ds))
    da = h * cs["alpha"]
    fd_a = (loss(cs["R"], cs["sig"], cs["alpha"] + da) -
            loss(cs["R"], cs["sig"], cs["alpha"] - da)) / (2 * da)
    gR = R.grad.cpu().numpy()[idx]
    gs = s.grad.cpu().numpy()[idx]
    fd_R, fd_s = np.array(fd_R), np.array(fd_s)
    assert np.abs(gR - fd_R).max() <= tol * np.abs(fd_R).max(), (gR, fd_R)
    assert np.abs(gs - fd_s).max() <= tol * np.abs(fd_s).max(), (gs, fd_s)
    assert abs(float(a.grad) - fd_a) <= tol * abs(fd_a), (float(a.grad), fd_a)


def test_adjoint_rejects_joint_and_bad_window(case):
    cs = case
    with pytest.raises(ValueError):
        WindowPowerModel(cs["pos"], cs["uct"], cs["bed"], [cs["surf"]],
                         [1.0, 3.15], [0.0, 10.0], window=(0, 999),
                         alpha_legs=(1,), corr_length=4.0, phasors=cs["ph"],
                         n_terms=40, **cs["common"])
