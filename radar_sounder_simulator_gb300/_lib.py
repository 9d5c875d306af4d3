"""ctypes binding of ``libsoundercuda.so`` (the C ABI in
``include/soundersim_gb300.h``).

The library is built in-tree (``radar_sounder_simulator_gb300.build``). There
is no fallback: if it cannot be loaded, every entry point raises.
"""

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsoundercuda.so")

SS_OK, SS_ERR_ARG, SS_ERR_CUDA, SS_ERR_UNSUPPORTED, SS_ERR_SCRATCH = range(5)
PREC = {"fp64": 0, "split": 1}
PATTERN = {"isotropic": 0, "dipole": 1, "array": 2, "array_tapered": 3,
           "finite_dipole": 4, "tabulated": 5}
ROUGH_NONE, ROUGH_GAUSS_FULL, ROUGH_GAUSS_AREA, ROUGH_EXP_AREA = range(4)
WIN_HANN, WIN_RECT = range(2)
PROJ = {None: 0, "EPSG:3413": 1, "EPSG:3031": 2}

_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)


class Facets(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "cx", "cy", "cz", "nx", "ny", "nz", "e1x", "e1y", "e1z", "e2x",
        "e2y", "e2z", "area", "gamma_f32", "gamma_f64", "sigma", "corr",
        "phasor", "diffuse_amp", "diffuse_phasor")] + [("n_facets", C.c_int32)]


class Traces(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("uct", C.c_void_p), ("pv", C.c_void_p),
                ("off", C.c_void_p), ("n_traces", C.c_int32),
                ("pv_len", C.c_int32)]


class Pattern(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n", C.c_int32), ("pa", C.c_void_p),
                ("pb", C.c_void_p)]


class Roughness(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_terms", C.c_int32),
                ("sigma", C.c_double), ("corr", C.c_double)]


class CoherentOpts(C.Structure):
    _fields_ = [("k", C.c_double), ("gamma", C.c_double), ("t0", C.c_double),
                ("dt", C.c_double), ("c", C.c_double),
                ("taper_s", C.c_double), ("n_samples", C.c_int32),
                ("block_size", C.c_int32), ("n_win", C.c_int32),
                ("split_sides", C.c_int32), ("interp_bins", C.c_int32),
                ("taper", C.c_int32), ("precision", C.c_int32)]


class Output(C.Structure):
    _fields_ = [("field_c128", C.c_void_p), ("field_c64", C.c_void_p),
                ("dropped", C.c_void_p)]


class Interface(C.Structure):
    _fields_ = [("table", C.c_void_p), ("ny", C.c_int32), ("nx", C.c_int32),
                ("coef", C.c_double * 6), ("mean_point", C.c_double * 3),
                ("mean_normal", C.c_double * 3)]


class RefractedOpts(C.Structure):
    _fields_ = [("n_crossed", C.c_int32), ("k_pad", C.c_int32),
                ("n_legs", C.c_int32), ("crossed", C.POINTER(Interface)),
                ("n_leg", C.POINTER(C.c_double)),
                ("eps_leg", C.POINTER(C.c_double)),
                ("att_leg", C.POINTER(C.c_double)),
                ("sigma_crossed", C.POINTER(C.c_double)),
                ("k0", C.c_double), ("gamma", C.c_double),
                ("t0", C.c_double), ("dt", C.c_double), ("c", C.c_double),
                ("taper_s", C.c_double), ("diffuse_exp", C.c_double),
                ("n_samples", C.c_int32), ("block_size", C.c_int32),
                ("n_win", C.c_int32), ("split_sides", C.c_int32),
                ("coherent", C.c_int32), ("joint", C.c_int32),
                ("joint_newton", C.c_int32), ("joint_backtrack", C.c_int32),
                ("taper", C.c_int32), ("precision", C.c_int32)]


# entry point name -> (restype, argtypes); the ABI surface the tests check
class WaveformOpts(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "n_traces", "n_samples", "n_lanes", "n_taps", "center", "power",
        "in_f64")]


class MultifreqOpts(C.Structure):
    _fields_ = [("f0", C.c_double), ("bandwidth", C.c_double),
                ("c", C.c_double), ("gamma", C.c_double),
                ("taper_s", C.c_double), ("n_freq", C.c_int32),
                ("freeze_amplitudes", C.c_int32), ("taper", C.c_int32),
                ("block_size", C.c_int32), ("n_win", C.c_int32),
                ("precision", C.c_int32)]


class AdjointIO(C.Structure):
    _fields_ = [("field", C.c_void_p), ("grad_power", C.c_void_p),
                ("bin_lo", C.c_int32), ("bin_hi", C.c_int32),
                ("alpha_mask", C.c_void_p), ("grad_gamma_db", C.c_void_p),
                ("grad_sigma", C.c_void_p), ("grad_alpha", C.c_void_p),
                ("scratch", C.c_void_p), ("scratch_bytes", C.c_size_t)]


class CoherentJob(C.Structure):
    _fields_ = [("opts", CoherentOpts), ("facets", Facets),
                ("traces", Traces), ("pattern", Pattern),
                ("rough", Roughness), ("out", Output)]


class BatchTuning(C.Structure):
    _fields_ = [("threads", C.c_int32), ("max_tb", C.c_int32),
                ("items_per_sm", C.c_int32), ("ctas_per_sm", C.c_int32)]


class IncoherentOpts(C.Structure):
    _fields_ = [("t0", C.c_double), ("dt", C.c_double), ("c", C.c_double),
                ("n_samples", C.c_int32), ("split_sides", C.c_int32)]


class IncoherentOutput(C.Structure):
    _fields_ = [("power", C.c_void_p), ("dropped", C.c_void_p)]


class FocusOpts(C.Structure):
    _fields_ = [("wavelength", C.c_double), ("aperture_m", C.c_double),
                ("c", C.c_double), ("n_traces", C.c_int32),
                ("n_bins", C.c_int32), ("window", C.c_int32),
                ("precision", C.c_int32), ("in_f64", C.c_int32)]


class FocusOutput(C.Structure):
    _fields_ = [("field_c128", C.c_void_p), ("field_c64", C.c_void_p),
                ("power", C.c_void_p)]


class Frame(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("R", C.c_double * 9)]


class DemGrid(C.Structure):
    _fields_ = [("dem", C.c_void_p), ("ny", C.c_int32), ("nx", C.c_int32),
                ("rows", C.c_void_p), ("cols", C.c_void_p),
                ("n_rows", C.c_int32), ("n_cols", C.c_int32),
                ("transform", C.c_double * 6), ("projection", C.c_int32),
                ("frame", Frame)]


class FacetOut(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "centers", "normals", "areas", "e1", "e2", "cell", "phase_keys")]


class TraceProductsOpts(C.Structure):
    _fields_ = [("t0", C.c_double), ("dt", C.c_double), ("c", C.c_double),
                ("n_samples", C.c_int32)]


class TraceProductsOut(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "nadir_index", "nadir_twtt", "first_index", "first_twtt")]


class RefractedJob(C.Structure):
    _fields_ = [("opts", RefractedOpts), ("target", Facets),
                ("traces", Traces), ("pattern", Pattern),
                ("rough", Roughness), ("out", Output)]


class RefractedBatchInfo(C.Structure):
    _fields_ = [("n_jobs", C.c_int32), ("path_class", C.c_int32),
                ("rough_kind", C.c_int32), ("plain", C.c_int32),
                ("ctas", C.c_int32), ("reserved", C.c_int32),
                ("n_items", C.c_int64), ("n_out", C.c_int64),
                ("n_words", C.c_int64), ("smem", C.c_uint64),
                ("fix_smem", C.c_uint64), ("table_offset", C.c_uint64),
                ("mask_offset", C.c_uint64)]


class BatchInfo(C.Structure):
    _fields_ = [("n_jobs", C.c_int32), ("precision", C.c_int32),
                ("rough_kind", C.c_int32), ("threads", C.c_int32),
                ("ctas", C.c_int32), ("reserved", C.c_int32),
                ("n_items", C.c_int64), ("n_out", C.c_int64),
                ("smem", C.c_uint64), ("table_offset", C.c_uint64)]


SIGNATURES = {
    "ss_coherent_scratch_bytes": (C.c_size_t, [C.POINTER(CoherentOpts),
                                               C.c_int32, C.c_int32]),
    "ss_coherent_fwd": (C.c_int, [C.POINTER(CoherentOpts), C.POINTER(Facets),
                                  C.POINTER(Traces), C.POINTER(Pattern),
                                  C.POINTER(Roughness), C.POINTER(Output),
                                  C.c_void_p, C.c_size_t, C.c_void_p]),
    "ss_coherent_fwd_noalloc": (C.c_int, [C.POINTER(CoherentOpts),
                                          C.POINTER(Facets), C.POINTER(Traces),
                                          C.POINTER(Pattern),
                                          C.POINTER(Roughness),
                                          C.POINTER(Output), C.c_void_p]),
    "ss_refracted_scratch_bytes": (C.c_size_t, [C.POINTER(RefractedOpts),
                                                C.c_int32, C.c_int32]),
    "ss_refracted_fwd": (C.c_int, [C.POINTER(RefractedOpts),
                                   C.POINTER(Facets), C.POINTER(Traces),
                                   C.POINTER(Pattern), C.POINTER(Roughness),
                                   C.POINTER(Output), C.c_void_p, C.c_size_t,
                                   C.c_void_p]),
    "ss_range_compress": (C.c_int, [C.POINTER(WaveformOpts), C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_range_compress_fft_scratch_bytes": (C.c_size_t,
                                            [C.POINTER(WaveformOpts)]),
    "ss_range_compress_fft": (C.c_int, [C.POINTER(WaveformOpts), C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_size_t, C.c_void_p]),
    "ss_range_compress_plan_bytes": (C.c_size_t, [C.POINTER(WaveformOpts),
                                                  C.c_int32]),
    "ss_range_compress_plan": (C.c_int, [C.POINTER(WaveformOpts), C.c_int32,
                                         C.c_void_p, C.c_void_p, C.c_size_t,
                                         C.c_void_p]),
    "ss_range_compress_apply": (C.c_int, [C.POINTER(WaveformOpts), C.c_int32,
                                          C.c_void_p, C.c_size_t, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    "ss_multifreq_scratch_bytes": (C.c_size_t, [C.POINTER(MultifreqOpts),
                                                C.c_int32, C.c_int32]),
    "ss_multifreq_response": (C.c_int, [C.POINTER(MultifreqOpts),
                                        C.POINTER(Facets), C.POINTER(Traces),
                                        C.POINTER(Roughness), C.c_void_p,
                                        C.c_void_p, C.c_size_t, C.c_void_p]),
    "ss_multifreq_synth": (C.c_int, [C.POINTER(MultifreqOpts), C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_int32, C.c_void_p, C.c_void_p]),
    "ss_refracted_adjoint_blocks": (C.c_int32, [C.c_int32]),
    "ss_refracted_adjoint_scratch_bytes": (C.c_size_t, [C.c_int32,
                                                        C.c_int32]),
    "ss_refracted_adjoint": (C.c_int, [C.POINTER(RefractedOpts),
                                       C.POINTER(Facets), C.POINTER(Traces),
                                       C.POINTER(Pattern),
                                       C.POINTER(Roughness),
                                       C.POINTER(AdjointIO), C.c_void_p]),
    "ss_coherent_batch_scratch_bytes": (C.c_size_t, [
        C.POINTER(CoherentJob), C.c_int32, C.POINTER(BatchTuning)]),
    "ss_coherent_batch_prepare": (C.c_int, [
        C.POINTER(CoherentJob), C.c_int32, C.POINTER(BatchTuning),
        C.c_void_p, C.c_size_t, C.POINTER(BatchInfo)]),
    "ss_refracted_batch_scratch_bytes": (C.c_size_t, [
        C.POINTER(RefractedJob), C.c_int32, C.POINTER(BatchTuning)]),
    "ss_refracted_batch_prepare": (C.c_int, [
        C.POINTER(RefractedJob), C.c_int32, C.POINTER(BatchTuning),
        C.c_void_p, C.c_size_t, C.POINTER(RefractedBatchInfo)]),
    "ss_refracted_batch_run": (C.c_int, [C.POINTER(RefractedBatchInfo),
                                         C.c_void_p, C.c_void_p]),
    "ss_coherent_batch_run": (C.c_int, [C.POINTER(BatchInfo), C.c_void_p,
                                        C.c_void_p]),
    "ss_incoherent_scratch_bytes": (C.c_size_t, [C.POINTER(IncoherentOpts),
                                                 C.c_int32, C.c_int32]),
    "ss_incoherent_fwd": (C.c_int, [C.POINTER(IncoherentOpts),
                                    C.POINTER(Facets), C.POINTER(Traces),
                                    C.POINTER(Pattern),
                                    C.POINTER(IncoherentOutput), C.c_void_p,
                                    C.c_size_t, C.c_void_p]),
    "ss_focused_sar_scratch_bytes": (C.c_size_t, [C.POINTER(FocusOpts)]),
    "ss_focused_sar": (C.c_int, [C.POINTER(FocusOpts), C.c_void_p,
                                 C.c_void_p, C.c_void_p,
                                 C.POINTER(FocusOutput), C.c_void_p,
                                 C.c_size_t, C.c_void_p]),
    "ss_scene_vertices": (C.c_int, [C.POINTER(DemGrid), C.c_void_p,
                                    C.c_void_p]),
    "ss_facets_from_vertices": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32,
                                          C.c_void_p, C.c_void_p,
                                          C.POINTER(FacetOut), C.c_void_p]),
    "ss_speckle_phasors_keyed": (C.c_int, [C.c_void_p, C.c_int64,
                                           C.c_uint64, C.c_void_p,
                                           C.c_void_p]),
    "ss_offset_centers": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Frame),
                                    C.c_double, C.c_void_p, C.c_void_p]),
    "ss_trace_products_scratch_bytes": (C.c_size_t, [C.c_int32, C.c_int32]),
    "ss_trace_products": (C.c_int, [C.POINTER(TraceProductsOpts), C.c_void_p,
                                    C.c_int32, C.c_void_p, C.c_int32,
                                    C.POINTER(TraceProductsOut), C.c_void_p,
                                    C.c_size_t, C.c_void_p]),
    "ss_fp32_fma_probe": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p,
                                    C.c_void_p]),
    "ss_mufu_probe": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p,
                                C.c_void_p]),
    "ss_fp64_fma_probe": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p,
                                    C.c_void_p]),
    "ss_version": (C.c_char_p, []),
    "ss_last_error": (C.c_char_p, []),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def lib():
    """Load (once) and return the CUDA library; raises when it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                f"{LIB_PATH} not built: run `python -m "
                "radar_sounder_simulator_gb300.build` (there is no CPU "
                "fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what):
    """Map a library status code to the reference's exception types."""
    if status == SS_OK:
        return
    msg = lib().ss_last_error().decode(errors="replace")
    if status in (SS_ERR_ARG, SS_ERR_UNSUPPORTED):
        raise ValueError(f"{what}: {msg}")
    raise RuntimeError(f"{what} failed (status {status}): {msg}")
