"""The surface split kernel's trace blocks on tracks that are not the
benchmark's straight, evenly spaced lines.

A block shares one double-float reference (its middle trace) when its
traces lie within 160 m of that trace and within 1 m of the block's straight
track line; each trace then adds N = 2 (lam q.u + q.eps) + |w|^2 with the
off-line part eps in float32. Sparser or bent blocks take a reference per
trace. Each case here is held to the split form's bounds against the FP64
form (relative L2 1e-4, 1e-3 rad and 0.01 dB over bins above -60 dB, the
same occupied bins) at 60 and 450 MHz:

* a straight track at 25 m (one reference per six-trace block);
* a sparse track at 120 m (blocks wider than 160 m: a reference per trace);
* a track wiggling 0.4 m across (blocks bent by ~0.06 m: the q.eps term);
* a track wiggling 10 m across (blocks bent by ~1.5 m: a reference per
  trace).
"""

import numpy as np
import pytest

from tests.util import field_errors

pytestmark = pytest.mark.gpu

C = 299792458.0


def _scene():
    from radar_sounder_simulator_gb300 import scenes
    rng = np.random.default_rng(31)
    return scenes.surface(96, 50.0, 30.0, 1000.0, 0.0, rng)


def _track(n, spacing, wiggle):
    x = (np.arange(n) - (n - 1) / 2.0) * spacing
    y = wiggle * np.sin(x / 97.0)
    pos = np.column_stack([x, y, np.full(n, 20000.0)])
    uct = np.tile([0.0, -1.0, 0.0], (n, 1))
    return pos, uct


@pytest.mark.parametrize("f0", [60e6, 450e6])
@pytest.mark.parametrize("spacing,wiggle", [(25.0, 0.0), (120.0, 0.0),
                                            (25.0, 0.4), (25.0, 10.0)])
def test_block_references_hold_the_bounds(f0, spacing, wiggle):
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
    f = _scene()
    pos, uct = _track(48, spacing, wiggle)
    bw = 0.15 * f0
    dt = 1.0 / (2.0 * bw)
    n = 2048
    t0 = scenes.window(pos, f.centers, n_samples=n, dt=dt)
    kw = dict(k=2 * np.pi * f0 / C, gamma=-0.279, t0=t0, dt=dt, n_samples=n,
              c=C, out_dtype=np.complex128, device="cuda")
    args = (pos, uct, f.centers, f.normals, f.areas, f.e1, f.e2)
    a, da = coherent_cluttergram(*args, **kw, precision="split")
    b, db = coherent_cluttergram(*args, **kw, precision="fp64")
    peak = np.abs(b).max()
    assert peak > 0
    floor = 1e-12 * peak
    assert np.array_equal(np.abs(a) > floor, np.abs(b) > floor)
    e = field_errors(a, b)
    assert e["rel_l2"] <= 1e-4 and e["phase_rad"] <= 1e-3 and \
        e["power_db"] <= 0.01, (spacing, wiggle, f0, e)
    np.testing.assert_allclose(da, db, rtol=1e-4, atol=1e-9 * peak ** 2)
