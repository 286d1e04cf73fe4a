"""GB300-native drop-in for vcfpop's Bayesian STRUCTURE clustering sweep.

The compute path is libvcfpop_structure.so (hand-written sm_103a CUDA behind
the C ABI in include/vcfpop_structure.h); this package is its Python binding,
build script and synthetic-data generator.
"""
from . import synth  # noqa: F401
