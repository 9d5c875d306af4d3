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

def _src():
    """The reference's ``src/soundersim`` directory, from the checkout named
    by the ``SOUNDERSIM_REF`` environment variable (required: there is no
    default location)."""
    root = os.environ.get("SOUNDERSIM_REF")
    if not root:
        raise RuntimeError("set SOUNDERSIM_REF to the soundersim checkout "
                           "(the directory holding src/soundersim)")
    return os.path.join(root, "src", "soundersim")


def load():
    """Return a namespace with the reference modules used by the fixtures."""
    SRC = _src()
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
