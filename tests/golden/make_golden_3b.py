"""Generate tests/golden/threeb_golden.npz: 3B fixtures computed by the reference.

For a few seeded 3B blocks (rfba_gb300.synth.threeb_block) the fixture stores
the inputs and the reference's own results, computed by its headers
(forward_algorithm.h, spot_with_background.hh, storm.h, conjugate_gradient_only.h)
compiled on the host by oracle/build_ref.sh and run here:
  * ``grad``  SpotNegProbabilityDiffWithSampledBackground at the start spot;
  * ``opt``   the spot after the reference's ConjugateGradientOnly<5> loop
              (multispot5.cc:1624-1636), with ``opt_it`` line searches.
The reference tree exists only in the build container, so this script runs
there; the committed fixture travels with the repository. Usage:

    python tests/golden/make_golden_3b.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import threeb as T  # noqa: E402

OUT = Path(__file__).resolve().parent / "threeb_golden.npz"

# (seed, samples, frames, mask shape, line searches); the shipped model, unit
# variance and z factor, the reference's motion limits with cg.max_motion 0.5
CASES = [(0, 3, 10, (6, 5, 5), 5), (1, 4, 16, (7, 7, 5), 5), (2, 2, 24, (5, 6, 6), 8)]


def motion_limit(mu: float = 3.5, sigma: float = 1.0, max_motion: float = 0.5) -> np.ndarray:
    return max_motion * np.array([np.sqrt((np.exp(sigma ** 2) - 1) * np.exp(2 * mu + sigma ** 2)), 1, 1, 1, 1])


def main() -> None:
    if T.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref3b_host.so not built: run oracle/build_ref.sh first")
    out = {}
    for k, (seed, S, F, shape, iters) in enumerate(CASES):
        bg, pix, px, spot = T.synthetic_block(seed, S, F, shape)
        grad = T.ref_spot_neg_prob_diff(bg, pix, px, spot)
        opt, it = T.ref_cg_optimise(bg, pix, px, spot, motion_limit(), iters)
        for name, v in (("bg", bg), ("pix", pix), ("px", px), ("spot", spot), ("grad", grad), ("opt", opt)):
            out[f"c{k}_{name}"] = v
        out[f"c{k}_iters"] = np.int64(iters)
        out[f"c{k}_opt_it"] = np.int64(it)
    out["ncases"] = np.int64(len(CASES))
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(CASES)} cases)")


if __name__ == "__main__":
    main()
