"""GB300-native 3D SRRF radiality (RFBA GradientCalc drop-in).

The compute path is librfba_srrf.so (hand-written sm_103a CUDA kernels behind
the C-ABI in include/rfba_srrf.h); this package is its Python front end plus
the synthetic data generator used by the benchmarks.
"""
from .srrf import (Block, Config, Context, RfbaError, SRRFConf, SRRFGetMag, SRRFGradientCalc,  # noqa: F401
                   SRRFGradientCalcGPU, blocks_dosplit, blocks_gradientcalc, lib, version)
