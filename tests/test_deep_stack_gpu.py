"""Deep interface stacks: the joint solve through 10 and 20 crossed
interfaces (firn layering; the reference's firn runs use 10/20/40 layers and
pad every joint target to a power-of-two bucket, simulate.py:253-260),
against the float64 oracle.

* the golden joint case (two crossed interfaces) padded with no-op air
  planes to 10 and 20 interfaces (multilayer.py:286-330);
* a firn-like stack of 10 and 20 rough layers over a bed, permittivity
  rising with depth.

FP64 form within 1e-9 of the oracle's peak (same occupied bins); split form
within relative L2 1e-4, 1e-3 rad and 0.01 dB above -60 dB.
"""

import numpy as np
import pytest

from oracle import refracted as oref
from radar_sounder_simulator_gb300 import scenes
from radar_sounder_simulator_gb300.multilayer import refracted_cluttergram
from tests.test_oracle_golden import refracted_case
from tests.util import field_errors

pytestmark = pytest.mark.gpu
C = 299792458.0


def _firn(n_layers, seed=21):
    rng = np.random.default_rng(seed)
    crossed = [scenes.surface(16, 20.0, 0.5, 100.0, 0.0, rng)]
    for i in range(1, n_layers):
        crossed.append(scenes.surface(16, 20.0, 0.2, 100.0, -4.0 * i, rng))
    bed = scenes.surface(16, 20.0, 2.0, 100.0, -4.0 * n_layers - 30.0, rng)
    eps = [1.0] + list(np.linspace(1.8, 3.15, n_layers))
    att = [0.0] + [10.0] * n_layers
    pos, uct = scenes.straight_track(4, 25.0, 400.0)
    kw = dict(mode="coherent", t0=2 * 370.0 / C, dt=1.0 / 100e6,
              n_samples=512, c=C, gamma=0.3, k0=2 * np.pi * 60e6 / C,
              refraction="joint")
    return pos, uct, bed, crossed, eps, att, kw


def _cases(golden):
    g = golden("refracted")
    out = {}
    for pad in (10, 20):
        pos, uct, tgt, crossed, e, a, kw = refracted_case(g, "joint2")
        out[f"pad{pad}"] = (pos, uct, tgt, crossed, e, a,
                            dict(kw, pad_to=pad))
    for n in (10, 20):
        out[f"firn{n}"] = _firn(n)
    return out


CASES = ["pad10", "pad20", "firn10", "firn20"]


@pytest.mark.parametrize("case", CASES)
def test_deep_stack_fp64_and_split_vs_oracle(golden, case):
    pos, uct, tgt, crossed, e, a, kw = _cases(golden)[case]
    ref, ref_drop = oref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                               **kw)
    scale = np.abs(ref).max()
    assert scale > 0
    got, drop = refracted_cluttergram(pos, uct, tgt, crossed, e, a, **kw,
                                      precision="fp64",
                                      out_dtype=np.complex128)
    assert np.array_equal(got != 0, ref != 0), "occupied bins"
    assert np.abs(got - ref).max() <= 1e-9 * scale
    np.testing.assert_allclose(drop, ref_drop, rtol=1e-5,
                               atol=1e-9 * scale ** 2)
    got32, _ = refracted_cluttergram(pos, uct, tgt, crossed, e, a, **kw,
                                     precision="split",
                                     out_dtype=np.complex128)
    err = field_errors(got32, ref)
    assert err["rel_l2"] <= 1e-4, err
    assert err["phase_rad"] <= 1e-3, err
    assert err["power_db"] <= 0.01, err
