"""Seeded per-particle subsampling (CPU): the library's selection of the K
kept points per particle equals the oracle's restatement of the rule, and
the rule has the properties the sensor update relies on -- K distinct scan
indices, one in each stratum of consecutive indices, reproducible per
(seed, particle), different across particles and seeds."""
import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import _native as N


def _lib_indices(seed, i, n, k):
    lib = N.lib()
    return np.array([lib.tsdfl_subsample_index(seed, i, n, k, j) for j in range(k)], np.uint32)


@pytest.mark.parametrize("n,k", [(2048, 256), (2048, 2048), (8192, 256), (1000, 333), (5, 3), (1, 1)])
def test_selection_equals_oracle_and_is_stratified(n, k):
    for seed in (0, 7, 2**63 + 5):
        for i in (0, 1, 999, 123456):
            got = _lib_indices(seed, i, n, k)
            want = O.subsample_indices(seed, i, n, k)
            assert np.array_equal(got, want)
            lo = (np.arange(k, dtype=np.uint64) * n // k).astype(np.int64)
            hi = (np.arange(1, k + 1, dtype=np.uint64) * n // k).astype(np.int64)
            assert np.all(got >= lo) and np.all(got < hi)   # one per stratum, hence distinct
    a = O.subsample_indices(3, 0, 2048, 256)
    assert not np.array_equal(a, O.subsample_indices(3, 1, 2048, 256))
    assert not np.array_equal(a, O.subsample_indices(4, 0, 2048, 256))


def test_selection_is_uniform_within_strata():
    """Over many particles every position of an 8-point stratum is taken about
    equally often."""
    counts = np.zeros(8)
    for i in range(4000):
        idx = O.subsample_indices(11, i, 2048, 256)
        counts += np.bincount(idx % 8, minlength=8)
    frac = counts / counts.sum()
    assert np.all(np.abs(frac - 0.125) < 0.005)


def test_invalid_arguments():
    lib = N.lib()
    assert lib.tsdfl_subsample_index(1, 0, 10, 11, 0) == 0xFFFFFFFF
    assert lib.tsdfl_subsample_index(1, 0, 10, 0, 0) == 0xFFFFFFFF
    assert lib.tsdfl_subsample_index(1, 0, 10, 5, 5) == 0xFFFFFFFF
