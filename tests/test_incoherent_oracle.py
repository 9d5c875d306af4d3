"""The incoherent oracle (float32 restatement of kernels/incoherent.py)
against the reference's own outputs (tests/golden/incoherent.npz, made by
tests/golden/make_golden.py from the reference source): per-pair bins equal
bit for bit, binned and dropped power within float32 summation error."""

import numpy as np

from oracle import incoherent as oi

C = 299792458.0
F32 = np.float32


def _case(g):
    surf = [g[f"surf_{k}"] for k in ("centers", "normals", "areas")]
    base = dict(t0=float(g["t0"]), dt=float(g["dt"]),
                n_samples=int(g["n_samples"]), c=C)
    pat = (str(g["ant_kind"]), g["ant_pv"], g["ant_pa"], g["ant_pb"])
    cases = {"iso": {}, "split": dict(split_sides=True),
             "dipole": dict(pattern=pat), "blocks": dict(block_size=100)}
    return surf, base, cases


def test_pair_bins_bit_exact(golden):
    g = golden("incoherent")
    surf, base, _ = _case(g)
    cen, nrm, area = (np.asarray(a, F32) for a in surf)
    for t in range(len(g["pos"])):
        _, r, _, _ = oi.pair_terms(g["pos"][t].astype(F32),
                                   g["uct"][t].astype(F32), cen, nrm, area)
        b = oi.bins(r, F32(base["t0"]), F32(base["dt"]), F32(C))
        np.testing.assert_array_equal(b, g["inc_pair_bins"][t])
    # the window cuts both ends: some pairs bin before it, some after
    assert g["inc_pair_bins"].min() < 0
    assert g["inc_pair_bins"].max() >= base["n_samples"]


def test_power_and_dropped_match_reference(golden):
    g = golden("incoherent")
    surf, base, cases = _case(g)
    for name, kw in cases.items():
        p, d = oi.incoherent_cluttergram(g["pos"], g["uct"], *surf, **base,
                                         **kw)
        ref, dref = g[f"inc_{name}_power"], g[f"inc_{name}_dropped"]
        assert p.dtype == np.float32 and p.shape == ref.shape, name
        np.testing.assert_array_equal(p > 0, ref > 0)
        assert np.linalg.norm(p - ref) <= 1e-6 * np.linalg.norm(ref), name
        assert (dref > 0).all()
        np.testing.assert_allclose(d, dref, rtol=1e-6)


def test_split_halves_sum_to_combined(golden):
    g = golden("incoherent")
    np.testing.assert_allclose(g["inc_split_power"].sum(-1),
                               g["inc_iso_power"], rtol=1e-5, atol=0)
