"""Generate tests/golden/gibbs_golden.npz: statistics of the reference's own
3B Gibbs sampler and free-energy estimate, for the GPU sampler's tests.

The reference's GibbsSampler2 with its MT19937 generator and the body of
NegativeFreeEnergy::compute_with_mask (RFBA Main/sampled_multispot.h,
multispot5.cc:335-405) run compiled on the host
(oracle/_ref/libref3b_gibbs_host.so from oracle/build_ref.sh). The GPU sampler
draws from the same distribution with a different random stream, so the
fixture holds distribution statistics: per spot and frame the fraction of
draws in each state from one long chain, and free-energy estimates for several
seeds. The reference tree exists only in the build container, so this script
runs there; the committed fixture travels with the repository. Usage:

    python tests/golden/make_golden_gibbs.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import gibbs_oracle as G  # noqa: E402


def main():
    from oracle import oracle as O
    from oracle import threeb as T3
    from rfba_gb300 import synth
    if O.build_ref() is None or not G.ref_available():
        raise SystemExit("reference sources not found; fixtures need the reference")
    out = {}
    # chain statistics: 3 spots, 30 frames
    pix, pixels, spots = synth.threeb_spots_block(21, 30, (9, 9, 7), 3)
    moff, midx = G.spot_masks(pixels, spots)
    si = G.spot_intensity(pixels, spots, 1.0)
    n = 40000
    st, _ = G.ref_run(pix, si, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, 1, n, 7)
    out.update(chain_pix=pix, chain_pixels=pixels, chain_spots=spots, chain_draws=np.int64(n),
               chain_freq=np.stack([(st == j).mean(0) for j in range(3)], -1))  # [K][F][3]
    # free energy: 2 spots, 20 frames, 200 thermodynamic samples, 16 seeds
    pix, pixels, spots = synth.threeb_spots_block(23, 20, (9, 9, 7), 2)
    moff, midx = G.spot_masks(pixels, spots)
    prior = (np.log(40.0), 0.5, 0.0, 0.1)
    vals = [G.ref_free_energy(pix, pixels, spots, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, 1.0, *prior, 200, 1,
                              seed)[0] for seed in range(1, 17)]
    out.update(fe_pix=pix, fe_pixels=pixels, fe_spots=spots, fe_prior=np.array(prior), fe_samples=np.int64(200),
               fe_values=np.array(vals))
    path = ROOT / "tests" / "golden" / "gibbs_golden.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path}: free energy {np.mean(vals):.3f} +- {np.std(vals, ddof=1):.3f}")


if __name__ == "__main__":
    main()
