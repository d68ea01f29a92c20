"""Generate tests/golden/golden.npz: parity fixtures pinned to the reference.

Inputs are crops of the reference's own test data (Test Data/Microbubule.tif,
Test Data/nucleus.tif: 16-bit ImageJ stacks, volume-major pages) and seeded
synthetic series. For each case the fixture stores:
  * ``ref``    the reference's output, computed by its own GradientCalc sources
               (kernel.cu + GradientCalc.cpp) compiled as host code by
               oracle/build_ref.sh and run here (FP32, the reference's
               arithmetic);
  * ``oracle`` the FP64 oracle's output (oracle/srrf_oracle.cpp), rounded to
               float32.
The reference tree exists only in the build container, so this script runs
there; the committed fixture travels with the repository. Usage:

    python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import json
import os
import struct
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1, intensity_w=1)


def read_tiff_stack(path: str) -> np.ndarray:
    """Pages of an uncompressed 8/16-bit TIFF as [page][y][x]."""
    b = open(path, "rb").read()
    end = "<" if b[:2] == b"II" else ">"
    if struct.unpack(end + "H", b[2:4])[0] != 42:
        raise ValueError("not a classic TIFF")
    off = struct.unpack(end + "I", b[4:8])[0]
    size = {1: 1, 3: 2, 4: 4}
    pages = []
    while off:
        n = struct.unpack(end + "H", b[off:off + 2])[0]
        tags = {}
        for i in range(n):
            e = b[off + 2 + 12 * i: off + 14 + 12 * i]
            tag, typ, cnt = struct.unpack(end + "HHI", e[:8])
            if typ not in size:
                continue
            nb = size[typ] * cnt
            data = e[8:8 + nb] if nb <= 4 else b[struct.unpack(end + "I", e[8:12])[0]:][:nb]
            tags[tag] = struct.unpack(end + {1: "B", 3: "H", 4: "I"}[typ] * cnt, data)
        w, h, bits = tags[256][0], tags[257][0], tags[258][0]
        if tags.get(259, (1,))[0] != 1:
            raise ValueError("compressed TIFF")
        dt = np.dtype(end + ("u2" if bits == 16 else "u1"))
        buf = b"".join(b[o:o + c] for o, c in zip(tags[273], tags[279]))
        pages.append(np.frombuffer(buf, dt, count=w * h).reshape(h, w).astype(dt.newbyteorder("=")))
        off = struct.unpack(end + "I", b[off + 2 + 12 * n: off + 6 + 12 * n])[0]
    return np.stack(pages)


def series_from_tiff(path: str, z_slices: int) -> np.ndarray:
    """[t][z][y][x] from a volume-major page stack (GenerateBlock.m:45-52)."""
    p = read_tiff_stack(path)
    t = p.shape[0] // z_slices
    return p[: t * z_slices].reshape(t, z_slices, p.shape[1], p.shape[2])


def synthetic(seed, T, D, H, W, emitters=10):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), emitters)
    return synth.render(scene, (W, H, D), seed, np.uint16)


def legacy_ref(x: np.ndarray, conf) -> np.ndarray:
    """The reference's SRRFGradientCalc (GradientCalc.cpp:169) run in a temp
    directory holding an SRRF.ini written from conf."""
    L = O.ref_lib()
    ini = (f"[SRRF]\nRingRadius={conf.ring_radius}\nMagnification={conf.mag[0]}\nAxesinRing={conf.axes_in_ring}\n"
           f"MainRange={conf.main_range}\nXRange={conf.x_range}\nYRange={conf.y_range}\nZRange={conf.z_range}\n"
           f"[Temproal]\nMethod={conf.method}\nIntegrate_Temporal_Correlations={conf.itc}\n"
           f"TRAC_ORDER={conf.trac_order}\n[Radiality]\nRemove_Positivity_Constraint={conf.remove_con}\n"
           f"Renormalize={conf.renormalize}\nGradient_Smoothing={conf.gradient_smooth}\n"
           f"[Weighting]\nIntensity_Weighting={conf.intensity_w}\n[Split]\nBlockSizeX={conf.block_size[0]}\n"
           f"BlockSizeY={conf.block_size[1]}\nBlockSizeZ={conf.block_size[2]}\n")
    T, D, H, W = x.shape
    m = conf.mag[0]
    img = np.ascontiguousarray(x, np.float32).copy()
    dims = np.array([W, H, D, T], np.int32)
    out = np.zeros((D * m, H * m, W * m), np.float32)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        Path(d, "SRRF.ini").write_text(ini)
        Path(d, ".\\SRRF.ini").write_text(ini)  # the reference opens ".\SRRF.ini"
        os.chdir(d)
        try:
            L.legacy_entry(O._p(img, O.ctypes.c_float), O._p(dims, O.ctypes.c_int), O._p(out, O.ctypes.c_float))
        finally:
            os.chdir(cwd)
    return out, ini


def main(ref_root: str | None = None):
    from oracle.refroot import reference_root
    ref_root = reference_root(ref_root)
    O.build()
    if O.build_ref(ref_root) is None:
        raise SystemExit("reference sources not found; fixtures need the reference")
    mb = series_from_tiff(os.path.join(ref_root, "Test Data", "Microbubule.tif"), 18)
    nu = series_from_tiff(os.path.join(ref_root, "Test Data", "nucleus.tif"), 15)
    crops = {
        "mb": mb[:, 4:12, 14:26, 14:26],   # 30 x 8 x 12 x 12
        "nu": nu[:, 3:11, 19:31, 19:31],   # 30 x 8 x 12 x 12
        "mb_big": mb[:, 2:12, 12:28, 12:28],  # 30 x 10 x 16 x 16 (legacy block split)
        "syn": synthetic(77, 20, 8, 10, 10),
    }
    cases = [
        ("mb_tra_m2", "mb", dict(mag=2, method=1, **SHIPPED)),
        ("mb_trac2_itc1_m3", "mb", dict(mag=3, method=3, itc=1, trac_order=2, **SHIPPED)),
        ("nu_trac4_itc0_m2", "nu", dict(mag=2, method=3, itc=0, trac_order=4, **SHIPPED)),
        ("nu_trm_m2", "nu", dict(mag=2, method=0, **SHIPPED)),
        ("nu_trppm_m2", "nu", dict(mag=2, method=2, **SHIPPED)),
        ("syn_trac3_itc1_nosmooth", "syn", dict(mag=2, method=3, itc=1, trac_order=3, gradient_smooth=0)),
        ("syn_renorm_poscon", "syn", dict(mag=2, method=1, renormalize=1, remove_con=1, **{
            k: v for k, v in SHIPPED.items()})),
    ]
    arrays = {}
    meta = []
    for name, arr in crops.items():
        arrays[f"in_{name}"] = np.ascontiguousarray(arr, np.uint16)
    for name, src, kw in cases:
        conf = O.make_conf(**kw)
        x = arrays[f"in_{src}"].astype(np.float32)
        ref = O.ref_block(x, conf)
        orc = O.srrf_region(x, conf)
        arrays[f"ref_{name}"] = ref
        arrays[f"oracle_{name}"] = orc.astype(np.float32)
        meta.append(dict(name=name, input=f"in_{src}", kind="block", conf=kw))
    # the reference's block split / put-back loop through its own INI reader
    kw = dict(mag=2, method=1, block_size=(10, 10, 10), **SHIPPED)
    conf = O.make_conf(**kw)
    x = arrays["in_mb_big"].astype(np.float32)
    ref, ini = legacy_ref(x, conf)
    orc = O.legacy(x, conf, fill=0.0)
    arrays["ref_legacy_mb_block10"] = ref
    arrays["oracle_legacy_mb_block10"] = orc.astype(np.float32)
    meta.append(dict(name="legacy_mb_block10", input="in_mb_big", kind="legacy", conf=kw, ini=ini))
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(meta)} cases)")


if __name__ == "__main__":
    main(*sys.argv[1:])
