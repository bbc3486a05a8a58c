"""Host side of the fitting harness (no GPU): configuration sets and sizes."""
import numpy as np

from examinimd_gb300 import fit


def test_config_sets_match_the_fitting_workload():
    snap = fit.snap_config_set(64)
    sizes = [len(x) for x, _ in snap]
    assert len(snap) == 64 and min(sizes) == 16 and max(sizes) == 1024
    for x, box in snap:
        assert np.all(x >= 0) and np.all(x < box)
        # strains within +-2% of the 3.1803 A cubic cell
        n = round((len(x) / 2) ** (1 / 3))
        assert np.all(np.abs(box / (n * 3.1803) - 1.0) <= 0.02 + 1e-12)
        assert np.all(box > 2 * 0.5 * 4.73442)  # one image per cutoff
    lj = fit.lj_config_set(16)
    sizes = [len(x) for x, _ in lj]
    assert min(sizes) == 500 and max(sizes) == 4000


def test_ncoeff_and_synthetic_beta():
    assert fit.ncoeffall_for(8) == 56  # 55 bispectrum components + constant
    b = fit.synthetic_beta(20261203, 56)
    assert b[0] == -8.0 and b.shape == (56,)
    np.testing.assert_array_equal(b, fit.synthetic_beta(20261203, 56))
