"""The C-ABI library builds, loads and exports every entry point that
include/soundersim_gb300.h declares (no compute: runs without a GPU)."""

import os
import re

from radar_sounder_simulator_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ss_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_header_symbols():
    build.build()
    L = _lib.lib()
    decl = declared_symbols()
    assert decl, "no entry points declared"
    for name in decl:
        assert hasattr(L, name), f"{name} declared but not exported"
    assert set(_lib.SIGNATURES) <= decl | {"ss_version", "ss_last_error"}
    assert b"sm_103a" in L.ss_version()


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the ABI structs have the C layout (sizes and field
    offsets), checked by compiling a probe against the header with gcc."""
    import ctypes as C
    import shutil
    import subprocess
    import pytest
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {"ss_facets": _lib.Facets, "ss_traces": _lib.Traces,
               "ss_pattern": _lib.Pattern, "ss_roughness": _lib.Roughness,
               "ss_coherent_opts": _lib.CoherentOpts,
               "ss_output": _lib.Output, "ss_interface": _lib.Interface,
               "ss_refracted_opts": _lib.RefractedOpts,
               "ss_waveform_opts": _lib.WaveformOpts,
               "ss_multifreq_opts": _lib.MultifreqOpts,
               "ss_adjoint_io": _lib.AdjointIO,
               "ss_coherent_job": _lib.CoherentJob,
               "ss_batch_tuning": _lib.BatchTuning,
               "ss_batch_info": _lib.BatchInfo,
               "ss_incoherent_opts": _lib.IncoherentOpts,
               "ss_incoherent_output": _lib.IncoherentOutput,
               "ss_focus_opts": _lib.FocusOpts,
               "ss_focus_output": _lib.FocusOutput,
               "ss_frame": _lib.Frame, "ss_dem_grid": _lib.DemGrid,
               "ss_facet_out": _lib.FacetOut,
               "ss_trace_products_opts": _lib.TraceProductsOpts,
               "ss_trace_products_out": _lib.TraceProductsOut}
    lines = ["#include <stdio.h>", "#include <stddef.h>",
             '#include "soundersim_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", '
                         f'offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", f"-I{os.path.join(ROOT, 'include')}", str(src),
                    "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in
               subprocess.run([str(exe)], capture_output=True, text=True,
                              check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(py, fname).offset, \
                f"{cname}.{fname}"


def test_c_program_links_and_calls_host_entry_points(tmp_path):
    """A plain C program includes the header, links libsoundercuda.so and
    calls entry points that need no GPU (build string, scratch sizing,
    argument validation) -- the binding a C or cgo caller would use."""
    import shutil
    import subprocess
    import pytest
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    build.build()
    libdir = os.path.dirname(_lib.LIB_PATH)
    src = tmp_path / "caller.c"
    src.write_text(r"""
#include <stdio.h>
#include <string.h>
#include "soundersim_gb300.h"
int main(void) {
  ss_incoherent_opts o;
  memset(&o, 0, sizeof o);
  o.t0 = 1e-5; o.dt = 1e-8; o.c = 299792458.0; o.n_samples = 128;
  size_t n = ss_incoherent_scratch_bytes(&o, 64, 100000);
  ss_focus_opts f;
  memset(&f, 0, sizeof f);
  f.n_traces = 10; f.n_bins = 100;
  size_t nf = ss_focused_sar_scratch_bytes(&f);
  int st = ss_incoherent_fwd(NULL, NULL, NULL, NULL, NULL, NULL, 0, NULL);
  printf("%s|%zu|%zu|%d|%s\n", ss_version(), n, nf, st, ss_last_error());
  return 0;
}
""")
    exe = tmp_path / "caller"
    subprocess.run(["gcc", f"-I{os.path.join(ROOT, 'include')}", str(src),
                    f"-L{libdir}", "-lsoundercuda", f"-Wl,-rpath,{libdir}",
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True,
                         check=True).stdout.strip().split("|")
    assert "sm_103a" in out[0]
    assert int(out[1]) > 0 and int(out[2]) == 10 * 8 + 100 * 16
    assert int(out[3]) == 1 and "null argument" in out[4]


def _null_call_cases():
    import ctypes as C
    for name, (res, args) in sorted(_lib.SIGNATURES.items()):
        if res is C.c_size_t or name in ("ss_version", "ss_last_error",
                                         "ss_refracted_adjoint_blocks"):
            continue
        yield name, args


def test_every_entry_point_rejects_null_arguments():
    """Each status-returning entry point answers null pointers with
    SS_ERR_ARG and a message, before any CUDA call, and the Python side maps
    that status to ValueError (the reference's exception type for argument
    errors). Sizes are 1, so an empty call cannot pass as a no-op. Runs only
    on a host without a GPU, where no call can reach a launch."""
    import ctypes as C
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("host-only check; the GPU suite covers device calls")
    build.build()
    L = _lib.lib()
    seen = 0
    for name, args in _null_call_cases():
        vals = [1 if a in (C.c_int32, C.c_int64, C.c_uint64, C.c_size_t)
                else 0.0 if a is C.c_double else None for a in args]
        st = getattr(L, name)(*vals)
        assert st == _lib.SS_ERR_ARG, (name, st)
        assert L.ss_last_error(), name
        with pytest.raises(ValueError):
            _lib.check(st, name)
        seen += 1
    assert seen >= 20


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """Without the built library every entry point raises: there is no CPU
    fallback to fall into."""
    import numpy as np
    import pytest
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(_lib.LibraryMissing, match="no CPU"):
        _lib.lib()
    c = np.array([[0.0, 0.0, 0.0]])
    plan = prepare_coherent(np.array([[0.0, 0.0, 100.0]]),
                            np.array([[0.0, -1.0, 0.0]]), c,
                            np.array([[0.0, 0.0, 1.0]]), np.ones(1),
                            np.array([[1.0, 0.0, 0.0]]),
                            np.array([[0.0, 1.0, 0.0]]), k=1.0, gamma=-0.3,
                            t0=0.0, dt=1e-8, n_samples=128, c=3e8,
                            device="cpu")
    with pytest.raises(_lib.LibraryMissing):
        plan.run()


def test_split_jobs_refuse_antenna_tables_above_shared_capacity():
    """The split kernels stage the antenna table in shared memory (up to
    256 floats: 128 samples of a tabulated pattern). A larger table is
    refused while the job is validated -- for the one-call and the batched
    entry points alike -- before any device work (the pointers here are
    placeholders that are never dereferenced)."""
    import ctypes as C
    L = _lib.lib()
    buf = (C.c_double * 4)()
    ptr = C.cast(buf, C.c_void_p)
    job = _lib.CoherentJob()
    job.opts.k, job.opts.c, job.opts.dt = 1.0, 3e8, 1e-8
    job.opts.n_samples, job.opts.block_size, job.opts.n_win = 64, 64, 1
    job.opts.precision = _lib.PREC["split"]
    job.facets.cx = job.facets.area = ptr
    job.facets.n_facets = 64
    job.traces.pos = job.traces.off = job.traces.pv = ptr
    job.traces.n_traces, job.traces.pv_len = 4, 3
    job.pattern.kind = 5  # SS_PAT_TABULATED
    job.pattern.pa = job.pattern.pb = ptr
    job.out.field_c128 = job.out.dropped = ptr
    for n, ok in ((128, True), (129, False)):
        job.pattern.n = n
        got = L.ss_coherent_batch_scratch_bytes(C.byref(job), 1, None)
        if ok:
            assert got > 0
        else:
            assert got == 0
            assert "antenna table too large" in L.ss_last_error().decode()
