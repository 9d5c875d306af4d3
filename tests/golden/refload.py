"""Import the reference's kernel modules from its source tree (fixture
generation only; this file reads the reference checkout and is never used on
the GPU host or by the product).

``soundersim/__init__.py`` pulls in xarray (absent here), so the package and
its ``kernels``/``compare`` sub-packages are registered as bare namespace
modules and only the leaf modules the coherent/refracted path needs are
executed, with ``jaxshim`` standing in for JAX.
"""

import importlib
import os
import sys
import types

from . import jaxshim

REF_ROOT = os.environ.get("SOUNDERSIM_REF", "/root/reference")
SRC = os.path.join(REF_ROOT, "src", "soundersim")


def load():
    """Return a namespace with the reference modules used by the fixtures."""
    jaxshim.install()
    for name, sub in (("soundersim", ""), ("soundersim.kernels", "kernels"),
                      ("soundersim.compare", "compare")):
        if name not in sys.modules or not hasattr(sys.modules[name],
                                                  "_shim_pkg"):
            mod = types.ModuleType(name)
            mod.__path__ = [os.path.join(SRC, sub) if sub else SRC]
            mod._shim_pkg = True
            sys.modules[name] = mod
    ns = types.SimpleNamespace()
    for attr, modname in (
            ("geometry", "soundersim.kernels.geometry"),
            ("coherent", "soundersim.kernels.coherent"),
            ("multilayer", "soundersim.kernels.multilayer"),
            ("roughness", "soundersim.roughness"),
            ("refraction", "soundersim.refraction"),
            ("refraction_joint", "soundersim.refraction_joint"),
            ("antenna", "soundersim.antenna"),
            ("physics", "soundersim.physics"),
            ("waveform", "soundersim.waveform"),
            ("multifreq", "soundersim.compare.multifreq"),
            ("brute_force", "soundersim.compare.brute_force"),
            ("gerekos", "soundersim.compare.gerekos"),
            ("scene", "soundersim.scene_light")):
        if modname == "soundersim.scene_light":
            ns.Facets = _facets_class()
            continue
        setattr(ns, attr, importlib.import_module(modname))
    return ns


def _facets_class():
    """``scene.Facets`` without importing scene.py (it needs pyproj): the
    refracted kernel only reads attributes, so a dataclass with the same
    fields (reference ``scene.py:80-101``) is enough."""
    from dataclasses import dataclass

    import numpy as np

    @dataclass
    class Facets:
        centers: np.ndarray
        normals: np.ndarray
        areas: np.ndarray
        e1: np.ndarray
        e2: np.ndarray
        cell: np.ndarray
        grid_shape: tuple
        phase_keys: np.ndarray = None

    return Facets
