"""CombineBlock.m on the GPU from the command line:

    python -m rfba_gb300.combine_cli --dims X Y Z --block BX BY BZ --border B \\
        [--zoom 10] [--sigma 3.5] [--psf-threshold 1000] [--noise-r 30] [--noise-rz 3] \\
        [--noise-threshold 70] RES_DIR OUT.tif

reads RES_DIR/res_i_j_k.txt for every doSplit block (the split parameters the
script loads from its .mat file: image size, block size, border), keeps each
block's spots as loadResult.m does, and writes the reconstruction as uint16 TIFF
pages (one per zoomed z slice, y rows, x columns) like the script's imwrite loop.
"""
from __future__ import annotations

import argparse
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--dims", type=int, nargs=3, required=True, metavar=("X", "Y", "Z"))
    ap.add_argument("--block", type=int, nargs=3, required=True, metavar=("BX", "BY", "BZ"))
    ap.add_argument("--border", type=int, required=True)
    ap.add_argument("--zoom", type=int, default=10)
    ap.add_argument("--sigma", type=float, default=3.5)
    ap.add_argument("--psf-threshold", type=float, default=1000.0)
    ap.add_argument("--noise-r", type=int, default=30)
    ap.add_argument("--noise-rz", type=int, default=3)
    ap.add_argument("--noise-threshold", type=int, default=70)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("res_dir")
    ap.add_argument("out")
    a = ap.parse_args(argv)
    from rfba_gb300 import srrf
    from rfba_gb300.tiff import write_tiff
    ctx = srrf.Context(a.device)
    try:
        vol, dropped = ctx.combine_blocks(a.res_dir, a.dims, a.block, a.border, a.zoom, a.sigma, a.psf_threshold,
                                          a.noise_r, a.noise_rz, a.noise_threshold)
    finally:
        ctx.close()
    write_tiff(a.out, vol)
    if dropped:
        print(f"{dropped} spots fell outside the zoomed grid", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
