"""Result cache keyed by the kernel version (the campaign driver's chunk
cache contract): a hit only when the metadata and the library build and
precision form all match (runs without a GPU: the library loads on any
host)."""

import numpy as np
import pytest

from radar_sounder_simulator_gb300 import build
from radar_sounder_simulator_gb300.cache import (ResultCache, kernel_version,
                                                 meta_key)


def test_cache_round_trip_and_invalidation(tmp_path):
    build.build()
    cache = ResultCache(tmp_path / "runs")
    meta = {"pass": "L1", "chunk": 3, "rows": [0, 511], "att": 10.0}
    calls = []

    def run():
        calls.append(1)
        return {"field": np.arange(6, dtype=np.complex64).reshape(2, 3),
                "dropped": np.ones(2, np.float32)}
    a = cache.get_or_run("L1_c3", meta, "split", run)
    b = cache.get_or_run("L1_c3", meta, "split", run)
    assert len(calls) == 1
    np.testing.assert_array_equal(a["field"], b["field"])
    # another precision form or changed metadata never hits
    assert cache.load("L1_c3", meta, "fp64") is None
    assert cache.load("L1_c3", {**meta, "att": 12.0}, "split") is None
    assert "sm_103a" in kernel_version("split")
    assert meta_key(meta, "split") != meta_key(meta, "fp64")
    with pytest.raises(ValueError):
        kernel_version("half")
