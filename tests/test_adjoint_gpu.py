"""Adjoint of windowed bed power against float64 central finite
differences of the oracle.

The reference has no gradient code (and ``jax.grad`` cannot run here), so
the gradients are pinned by central differences of the float64 oracle
forward (``oracle.refracted``, the restated multilayer.py:594-770) on the
same float32-quantised facets: relative step 2^-13 (~1.2e-4) on 64 seeded
facets per parameter kind (reflectivity in dB, rms height) plus the
attenuation rate. With the FP64 forward every checked entry agrees within
1e-4 of its own finite difference, with an absolute floor of 1e-5 of the
largest checked gradient of its kind (entries five orders below the largest
carry no float32-meaningful digits). With the split forward the field that
weights each pair's derivative carries ~1e-5 relative error (more in the
weakest bins), so its entries are held to 2e-4 with a floor of 1e-4 of the
largest. Both refraction paths: a bed under one interface (sequential
chain) and a bed under two (joint solve).
"""

import numpy as np
import pytest
import torch

from oracle import refracted as orf
from radar_sounder_simulator_gb300 import scenes
from radar_sounder_simulator_gb300.adjoint import WindowPowerModel, db_misfit

pytestmark = pytest.mark.gpu
C = 299792458.0
N_CHECK = 64
BOUNDS = {"fp64": (1e-4, 1e-5), "split": (2e-4, 1e-4)}  # (relative, floor)


def _q10(x):
    """Round to 10 significant bits so x (1 +- 2^-13) is exact in float32."""
    e = np.floor(np.log2(np.abs(x)))
    return np.round(x / 2.0 ** (e - 9)) * 2.0 ** (e - 9)


@pytest.fixture(scope="module", params=["sequential", "joint"])
def case(request):
    rng = np.random.default_rng(11)
    surf = scenes.surface(20, 25.0, 2.0, 200.0, 0.0, rng)
    mid = scenes.surface(20, 25.0, 1.0, 200.0, -80.0, rng)
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
    if request.param == "joint":
        crossed, eps, att = [surf, mid], [1.0, 2.9, 3.15], [0.0, 10.0, 10.0]
        alpha_legs = (1, 2)
    else:
        crossed, eps, att = [surf], [1.0, 3.15], [0.0, 10.0]
        alpha_legs = (1,)
    return dict(refraction=request.param, crossed=crossed, eps=eps, att=att,
                alpha_legs=alpha_legs, bed=bed, pos=pos, uct=uct, ph=ph, R=R,
                sig=sig, alpha=10.0, common=common, n=n)


def oracle_power(cs, R, sig, alpha):
    att = [alpha if m in cs["alpha_legs"] else v
           for m, v in enumerate(cs["att"])]
    out, _ = orf.refracted_cluttergram(
        cs["pos"], cs["uct"], cs["bed"], cs["crossed"], cs["eps"], att,
        mode="coherent", gamma=10.0 ** (R / 20.0),
        roughness=(sig, 4.0, cs["ph"], 40, "exponential"), d_phi_area=True,
        taper_s=0.05, refraction=cs["refraction"], **cs["common"])
    return (np.abs(out) ** 2).sum(axis=1)


def _check(name, got, fd, forward):
    rel, fl = BOUNDS[forward]
    floor = fl * np.abs(fd).max()
    bad = np.abs(got - fd) > rel * np.abs(fd) + floor
    assert not bad.any(), (name, got[bad], fd[bad])


@pytest.fixture(scope="module")
def fd(case):
    """Target power and float64 central differences of the misfit on the
    seeded parameters (shared by both forward forms)."""
    cs = case
    rng = np.random.default_rng(5)
    R_hat = cs["R"] + rng.standard_normal(cs["n"])
    s_hat = _q10(cs["sig"] * np.exp(0.1 * rng.standard_normal(cs["n"])))
    P_hat = oracle_power(cs, R_hat, s_hat, cs["alpha"] + 1.0)

    def loss(Rv, sv, av):
        Pv = oracle_power(cs, Rv, sv, av)
        return float(((10 * np.log10(Pv) - 10 * np.log10(P_hat)) ** 2).sum())

    h = 2.0 ** -13
    idx = rng.choice(cs["n"], size=N_CHECK, replace=False)
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
    return dict(P_hat=P_hat, idx=idx, R=np.array(fd_R), s=np.array(fd_s),
                a=fd_a, P64=oracle_power(cs, cs["R"], cs["sig"],
                                         cs["alpha"]))


@pytest.mark.parametrize("forward", ["fp64", "split"])
def test_adjoint_matches_central_differences(case, fd, forward):
    """The adjoint recomputes each pair in split precision and weights it by
    the forward field: float64 with the FP64 forward, split precision
    (P within ~2e-5 on this rough scene, held to 1e-4) with the split
    forward."""
    cs = case
    model = WindowPowerModel(
        cs["pos"], cs["uct"], cs["bed"], cs["crossed"], cs["eps"],
        cs["att"], window=(0, 256), alpha_legs=cs["alpha_legs"],
        corr_length=4.0, phasors=cs["ph"], n_terms=40,
        refraction=cs["refraction"], precision=forward, **cs["common"])
    dev = model.device
    P_hat = torch.as_tensor(fd["P_hat"], device=dev)
    R = torch.tensor(cs["R"], device=dev, requires_grad=True)
    s = torch.tensor(cs["sig"], device=dev, requires_grad=True)
    a = torch.tensor(cs["alpha"], dtype=torch.float64, device=dev,
                     requires_grad=True)
    P = model.power(R, s, a)
    assert np.abs(P.detach().cpu().numpy() / fd["P64"] - 1).max() < (
        1e-9 if forward == "fp64" else 1e-4)
    db_misfit(P, P_hat).backward()
    idx = fd["idx"]
    _check("reflectivity", R.grad.cpu().numpy()[idx], fd["R"], forward)
    _check("rms height", s.grad.cpu().numpy()[idx], fd["s"], forward)
    assert abs(float(a.grad) - fd["a"]) <= BOUNDS[forward][0] * abs(
        fd["a"]), (float(a.grad), fd["a"])


def test_adjoint_rejects_bad_window(case):
    cs = case
    with pytest.raises(ValueError):
        WindowPowerModel(cs["pos"], cs["uct"], cs["bed"], cs["crossed"],
                         cs["eps"], cs["att"], window=(0, 999),
                         alpha_legs=cs["alpha_legs"], corr_length=4.0,
                         phasors=cs["ph"], n_terms=40,
                         refraction=cs["refraction"], **cs["common"])
