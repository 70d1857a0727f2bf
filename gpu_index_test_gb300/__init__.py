"""GB300-native strobealign seeding → index lookup → NAM path.

The product is libgbsa.so (CUDA kernels for sm_103a behind the C-ABI declared in
include/gbsa.h).  This package holds its sources (csrc/), the build recipe, a
ctypes binding of the C-ABI (native.py), and the seeded synthetic data generator
(synth.py).
"""
