"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Input generation for the benchmark and the tests only: nothing in the library (matflat_gb300/)
imports it, and it loads no library file of the product.  `synth` holds the generators; the
host helper `libworkloads_synth.so` (built from synth.c by `build`) gives the GPU path and the
CPU oracle identical bytes.
"""
