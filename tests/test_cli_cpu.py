"""rfba-srrf (the RFBA.bat --srrf_only step) on the CPU: TIFF pages parsed in
both byte orders, 8 and 16 bit, one or several strips per page; unsupported
files and mismatched volumes rejected. No GPU is touched (--info)."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.tiffio import write_tiff

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "rfba_gb300" / "_lib" / "rfba-srrf"


@pytest.fixture(scope="module")
def cli(built_lib):
    from rfba_gb300 import build as B
    B.build_cli()
    assert CLI.exists()
    return str(CLI)


@pytest.mark.parametrize("dtype,big,rps", [(np.uint16, False, None), (np.uint16, True, 3), (np.uint8, False, 4),
                                          (np.uint8, True, None)])
def test_info_reads_pages(cli, tmp_path, dtype, big, rps):
    rng = np.random.default_rng(1)
    vol = rng.integers(0, np.iinfo(dtype).max, size=(5, 7, 9)).astype(dtype)
    p = tmp_path / "v.tif"
    write_tiff(p, vol, big_endian=big, rows_per_strip=rps)
    r = subprocess.run([cli, "--info", str(p)], capture_output=True, text=True, check=True)
    name, w, h, d, bits, s = r.stdout.rsplit(maxsplit=5)
    assert (int(w), int(h), int(d), int(bits)) == (9, 7, 5, 8 * np.dtype(dtype).itemsize)
    assert float(s) == float(vol.astype(np.float64).sum())


def test_rejects_mismatched_and_bad_files(cli, tmp_path):
    a, b = tmp_path / "a.tif", tmp_path / "b.tif"
    write_tiff(a, np.zeros((3, 4, 4), np.uint16))
    write_tiff(b, np.zeros((3, 4, 5), np.uint16))
    r = subprocess.run([cli, "--info", str(a), str(b)], capture_output=True, text=True)
    assert r.returncode == 1 and "same size" in r.stderr
    c = tmp_path / "c.tif"
    c.write_bytes(b"not a tiff at all")
    r = subprocess.run([cli, "--info", str(c)], capture_output=True, text=True)
    assert r.returncode == 1 and "not a TIFF" in r.stderr
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 2


def test_reads_reference_test_data(cli):
    from oracle.refroot import reference_root
    p = Path(reference_root(), "Test Data", "Microbubule.tif")
    if not p.exists():
        pytest.skip("reference test data not present")
    r = subprocess.run([cli, "--info", str(p)], capture_output=True, text=True, check=True)
    f = r.stdout.rsplit(maxsplit=5)
    assert f[1:5] == ["40", "40", "540", "16"]
