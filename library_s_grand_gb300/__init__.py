"""GB300-native GRAND decoder (drop-in for CarolinaBoavida/Library_S_GRAND).

The product is ``libgranddecoder.so`` (C ABI in include/grand_decoder.h), built
from ``csrc/`` for sm_103a by ``library_s_grand_gb300.build``.  This package
holds the ctypes binding that mirrors the upstream Python helpers
(``capi``), seeded synthetic codes and shots (``synth``), and the build step.
"""
from .capi import (  # noqa: F401
    GrandDecodeOutputs,
    GrandDecoderConfig,
    GrandDecoderResult,
    RESULT_DTYPE,
    load_library,
    run_grand_ML_shots_cln,
    run_grand_prob_shots_cc,
    run_grand_prob_shots_cln,
    run_grand_shots_cc,
    run_grand_shots_cln,
)

__version__ = "0.1.0"
