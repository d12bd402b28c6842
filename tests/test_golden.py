"""The CPU oracle against golden vectors produced by the REFERENCE's own
CUDA driver (src/__GpuDriver.cu, reel = double) on a GB300, by
tests/golden/make_ref_golden.py: _getAmplitudes (sample and hold, window 4,
config-2 and config-1 shaped systems), _getTrajectory and _getGradient.

The reference sums the nonlinear terms with atomicAdd in an unspecified
order, so agreement is to rounding: 1e-10 relative (FP64), the bound the
FP64 path is held to."""
import glob
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from pasif_gb300.system import Pattern

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


def pattern(z, pre, n_sp=None):
    return Pattern(n=int(z[pre + "n"]), k_ptr=z[pre + "k_ptr"], k_col=z[pre + "k_col"], g_idx=z[pre + "g"],
                   l_idx=z[pre + "l"], p_idx=z[pre + "p"], f_idx=z[pre + "f"], n_sp=n_sp or 0)


def test_fixtures_present():
    assert len(FILES) >= 7


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[4:-4] for f in FILES])
def test_oracle_matches_reference_driver(path):
    z = np.load(path)
    fp = pattern(z, "f_")
    fv = z["f_vals"]
    W = int(z["W"])
    im = z["im"].reshape(2, W) if W else None
    h, N, task = float(z["h"]), int(z["N"]), int(z["task"])
    if task == 0:
        got = O.get_amplitudes(fp, fv, z["x0"], z["x"], h, N, W, im)
    elif task == 1:
        got = O.get_trajectory(fp, fv, z["x0"], z["x"], h, N, int(z["save"]), W, im)
    else:
        bp = pattern(z, "b_", n_sp=fp.n)
        got = O.get_gradient(fp, fv, z["x0"], bp, z["b_vals"], z["a0"], z["x"], h, N, int(z["save"]), W, im)
    ref = z["out"]
    assert got.shape == ref.shape
    # a diverging copy must diverge in both (same non-finite entries)
    np.testing.assert_array_equal(np.isfinite(got), np.isfinite(ref))
    ok = np.isfinite(ref)
    assert ok.sum() >= 0.5 * ref.size
    g, r = got[ok], ref[ok]
    scale = np.maximum(np.abs(r), 1e-12 * np.abs(r).max() + 1e-300)
    rel = np.abs(g - r) / scale
    assert rel.max() <= 1e-10, (rel.max(), np.argmax(rel))
