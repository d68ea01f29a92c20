"""rfba-srrf end to end: per-volume TIFF files -> global-std normalisation ->
SRRFGradientCalc with ./SRRF.ini -> NaN/negative clamp -> ./SRRF.raw, against
the same steps with the FP64 oracle's GradientCalc loop."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.parity import rel_linf
from tests.tiffio import write_tiff

pytestmark = pytest.mark.gpu
CLI = Path(__file__).resolve().parents[1] / "rfba_gb300" / "_lib" / "rfba-srrf"


def _normalise(x):
    """storm_imagery.cc:358-416 with skip=1, fixed_scaling=0: double sums of the
    voxels and of their float squares, mean/variance returned as floats."""
    xf = x.astype(np.float32)
    s = float(np.sum(xf.astype(np.float64)))
    s2 = float(np.sum((xf * xf).astype(np.float64)))
    area = float(xf.size)
    var = np.float64(np.float32(s2 / area - (s / area) ** 2))
    return (xf.astype(np.float64) / np.sqrt(var)).astype(np.float32)


@pytest.mark.parametrize("method", [1, 3])
def test_srrf_only_writes_srrf_raw(oracle_mod, tmp_path, method):
    from rfba_gb300 import build as B, synth
    B.build_cli()
    O = oracle_mod
    T, shape = 6, (20, 18, 14)
    scene = synth.make_scene(31, T, shape, 30)
    x = synth.render(scene, shape, 31, np.uint16)
    files = []
    for t in range(T):
        p = tmp_path / f"cell{t}.tif"
        write_tiff(p, x[t], big_endian=bool(t % 2))
        files.append(str(p))
    conf = O.make_conf(mag=2, method=method, itc=0, trac_order=2, gradient_smooth=1, main_range=1, x_range=1,
                       y_range=1, z_range=1, block_size=(12, 12, 12))
    ini = (f"[SRRF]\nRingRadius=0.5\nMagnification=2\nAxesinRing=6\nMainRange=1\nXRange=1\nYRange=1\nZRange=1\n"
           f"[Temproal]\nMethod={method}\nIntegrate_Temporal_Correlations=0\nTRAC_ORDER=2\n"
           f"[Radiality]\nRemove_Positivity_Constraint=0\nRenormalize=0\nGradient_Smoothing=1\n"
           f"[Weighting]\nIntensity_Weighting=1\n[Split]\nBlockSizeX=12\nBlockSizeY=12\nBlockSizeZ=12\n")
    (tmp_path / "SRRF.ini").write_text(ini)
    subprocess.run([str(CLI), "--srrf_only", "1", "--save_spots", "resdummy.txt", "--log_ratios", "markupdummy.tif",
                    *files], cwd=tmp_path, check=True, capture_output=True)
    raw = np.fromfile(tmp_path / "SRRF.raw", np.float32)
    D, H, W = x.shape[1:]
    assert raw.size == D * H * W * 8
    got = raw.reshape(D * 2, H * 2, W * 2)
    exp = O.legacy(_normalise(x), conf)
    exp = np.where(np.isnan(exp) | (exp < 0), 0.0, exp)
    assert np.all(np.isfinite(got)) and np.all(got >= 0)
    e = rel_linf(got, exp)
    print(f"[cli] SRRF.raw method {method}: rel L-inf vs FP64 oracle {e:.2e}")
    assert e < (1e-5 if method == 1 else 1e-4)
