"""ORACLE / TEST INFRASTRUCTURE ONLY.

The checker for the GB300 ARD time step: a C restatement of the reference's
algorithm (ard_oracle.c, float and double), a Python restatement of its scene
setup (scene_oracle.py), the FFTW-compatible DCT both use (dct_fft.c) and the
recipe that builds the reference itself headless (ref_build/).  Only tests/,
the smoke check and bench.py's CPU-baseline leg may import it; the product
never does.
"""
