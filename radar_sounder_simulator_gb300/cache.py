"""Result cache keyed by the kernel version.

The campaign driver of soundersim keeps each simulated chunk as
``<rid>.npz`` with a ``<rid>.json`` sidecar whose ``meta_key`` is the
sorted-key JSON of the chunk's metadata, including the kernel version
(tools/run_basal_clutter.py:1466-1505 and :2161-2205, with
``soundersim.kernels.KERNEL_VERSION``); a chunk is reused only when the key
matches. This module keeps that contract for results of this library: the
version word is the CUDA library's build string plus the precision form,
so results from another build or precision are never served.
"""

import json
from pathlib import Path

import numpy as np

from . import _lib


def kernel_version(precision):
    """Version word of this library for a precision form."""
    if precision not in _lib.PREC:
        raise ValueError(f"unknown precision {precision!r}")
    return f"{_lib.lib().ss_version().decode()} {precision}"


def meta_key(meta, precision):
    """The sorted-key JSON that identifies a result."""
    return json.dumps({**meta, "kernel": kernel_version(precision)},
                      sort_keys=True)


class ResultCache:
    """``<root>/<rid>.npz`` arrays with a ``<rid>.json`` sidecar."""

    def __init__(self, root):
        self.root = Path(root)

    def _paths(self, rid):
        return self.root / f"{rid}.json", self.root / f"{rid}.npz"

    def load(self, rid, meta, precision):
        """The stored arrays when the sidecar's key matches, else None."""
        jp, npz = self._paths(rid)
        if not (jp.exists() and npz.exists()):
            return None
        doc = json.loads(jp.read_text())
        if doc.get("meta_key") != meta_key(meta, precision):
            return None
        with np.load(npz) as z:
            return {k: z[k] for k in z.files}

    def save(self, rid, meta, precision, **arrays):
        self.root.mkdir(parents=True, exist_ok=True)
        jp, npz = self._paths(rid)
        np.savez(npz, **arrays)
        jp.write_text(json.dumps({"meta_key": meta_key(meta, precision),
                                  "meta": meta}, indent=1) + "\n")

    def get_or_run(self, rid, meta, precision, run):
        """Cached arrays for ``rid``, or ``run()`` (a dict of arrays),
        stored and returned."""
        hit = self.load(rid, meta, precision)
        if hit is not None:
            return hit
        arrays = run()
        self.save(rid, meta, precision, **arrays)
        return arrays
