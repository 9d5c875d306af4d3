"""ss_coherent_fwd_noalloc: the surface facet sum for callers that cannot
allocate device memory (their GPU memory belongs to another allocator, or
they must not allocate once running), served from a fixed scratch array in
the library. Checked through the C ABI against ss_coherent_fwd on the same
staged inputs, on two calls in a row (the array is shared and keeps the
previous call's partials), and for its clear rejection of sizes beyond the
array. Collected last so a failure here leaves every other test run."""

import ctypes as C

import numpy as np
import pytest

from tests.util import facets_from, field_errors

pytestmark = pytest.mark.gpu
LIGHT = 299792458.0


def _call_noalloc(plan, field, dropped):
    from radar_sounder_simulator_gb300 import _lib
    import torch
    out = _lib.Output(field.data_ptr(), None, dropped.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    return _lib.lib().ss_coherent_fwd_noalloc(
        C.byref(plan.opts), C.byref(plan.fst), C.byref(plan.tr),
        C.byref(plan.pst), C.byref(plan.rst), C.byref(out),
        C.c_void_p(stream))


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_noalloc_matches_scratch_entry_point(golden, precision):
    import torch
    from radar_sounder_simulator_gb300 import _lib
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    g = golden("coherent")
    f = facets_from(g, "surf")
    plan = prepare_coherent(
        g["pos"], g["uct"], f.centers, f.normals, f.areas, f.e1, f.e2,
        k=float(g["k"]), gamma=-0.279, t0=float(g["t0"]), dt=float(g["dt"]),
        n_samples=int(g["n_samples"]), c=LIGHT, split_sides=True,
        roughness=(0.3, 4.0, g["phasors"], 40), precision=precision)
    ref_f, ref_d = plan.run()
    ref = torch.view_as_complex(ref_f.contiguous()).cpu().numpy()
    for _ in range(2):
        field = torch.full_like(ref_f, float("nan"))
        dropped = torch.full_like(ref_d, float("nan"))
        st = _call_noalloc(plan, field, dropped)
        _lib.check(st, "ss_coherent_fwd_noalloc")
        torch.cuda.synchronize()
        got = torch.view_as_complex(field.contiguous()).cpu().numpy()
        assert np.isfinite(got).all()
        if precision == "fp64":
            assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
        else:
            err = field_errors(got, ref)
            assert err["rel_l2"] <= 1e-4 and err["phase_rad"] <= 1e-3
            assert err["power_db"] <= 0.01
        np.testing.assert_allclose(dropped.cpu().numpy(),
                                   ref_d.cpu().numpy(), rtol=1e-5,
                                   atol=1e-12)


def test_noalloc_rejects_sizes_beyond_its_array():
    """3000 traces x 2048 bins of float64 partials exceed the 64 MiB array:
    the call must refuse with SS_ERR_SCRATCH before queueing any work."""
    import torch
    from radar_sounder_simulator_gb300 import _lib
    dev = torch.device("cuda")
    T, N = 3000, 64
    pos = torch.zeros((T, 3), dtype=torch.float64, device=dev)
    off = torch.zeros(T, dtype=torch.int32, device=dev)
    soa = torch.zeros((13, N), dtype=torch.float32, device=dev)
    fac = _lib.Facets()
    for j, nm in enumerate(("cx", "cy", "cz", "nx", "ny", "nz", "e1x", "e1y",
                            "e1z", "e2x", "e2y", "e2z", "area")):
        setattr(fac, nm, soa.data_ptr() + 4 * N * j)
    fac.n_facets = N
    tr = _lib.Traces(pos.data_ptr(), pos.data_ptr(), None, off.data_ptr(), T,
                     0)
    opts = _lib.CoherentOpts(1.0, -0.3, 0.0, 1e-8, LIGHT, 0.0, 2048, 64, 1, 0,
                             0, 0, _lib.PREC["fp64"])
    field = torch.empty((T, 2048, 2), dtype=torch.float64, device=dev)
    dropped = torch.empty(T, dtype=torch.float64, device=dev)
    out = _lib.Output(field.data_ptr(), None, dropped.data_ptr())
    st = _lib.lib().ss_coherent_fwd_noalloc(
        C.byref(opts), C.byref(fac), C.byref(tr), None, None, C.byref(out),
        None)
    assert st == _lib.SS_ERR_SCRATCH
    assert b"SS_NOALLOC_SCRATCH_BYTES" in _lib.lib().ss_last_error()
