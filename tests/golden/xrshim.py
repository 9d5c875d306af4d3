"""Minimal stand-in for the parts of ``xarray`` that soundersim's
``processing.focused_sar`` touches (fixture generation only; xarray is not
installed here). ``Dataset`` holds named ``DataArray``s (data variables and
coordinates) and attrs; ``DataArray`` holds dims, values and attrs. Only
the calls focused_sar makes are provided: attribute and item access,
``dims``, ``values``, ``attrs``, ``transpose``, ``sizes``, ``copy`` and
item assignment from a ``(dims, values, attrs)`` tuple.
"""

import copy
import sys
import types


class DataArray:
    def __init__(self, dims, values, attrs=None):
        self.dims = tuple(dims)
        self.values = values
        self.attrs = dict(attrs or {})

    def transpose(self, *dims):
        perm = [self.dims.index(d) for d in dims]
        return DataArray(dims, self.values.transpose(perm), self.attrs)


class Dataset:
    def __init__(self, data_vars=None, coords=None, attrs=None):
        self._vars = {}
        self._coords = {}
        for k, v in (data_vars or {}).items():
            self._vars[k] = _as_array(v, k)
        for k, v in (coords or {}).items():
            self._coords[k] = _as_array(v, k)
        self.attrs = dict(attrs or {})

    @property
    def data_vars(self):
        return dict(self._vars)

    @property
    def coords(self):
        return dict(self._coords)

    @property
    def sizes(self):
        out = {}
        for a in list(self._vars.values()) + list(self._coords.values()):
            for d, n in zip(a.dims, a.values.shape):
                out[d] = n
        return out

    def __contains__(self, name):
        return name in self._vars or name in self._coords

    def __getitem__(self, name):
        return self._vars[name] if name in self._vars else self._coords[name]

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        try:
            return self[name]
        except KeyError:
            raise AttributeError(name) from None

    def __setitem__(self, name, value):
        self._vars[name] = _as_array(value, name)

    def copy(self):
        return copy.deepcopy(self)


def _as_array(v, name):
    if isinstance(v, DataArray):
        return v
    if not isinstance(v, tuple):      # a bare array: the dimension coord
        return DataArray((name,), v)
    dims, values, *rest = v
    if isinstance(dims, str):
        dims = (dims,)
    return DataArray(dims, values, rest[0] if rest else None)


def install():
    mod = types.ModuleType("xarray")
    mod.Dataset = Dataset
    mod.DataArray = DataArray
    sys.modules["xarray"] = mod
    return mod
