"""GB300-native integral-equation forward solve of extrEMe (prisae/extreme).

The compute path lives in ``libegx.so`` (hand-written sm_103a CUDA behind the
C ABI of ``include/egx.h``); :mod:`extreme_gb300.egx` binds it and
:mod:`extreme_gb300.forward` mirrors the reference's forward-solver classes.
"""
__version__ = "0.1.0"
