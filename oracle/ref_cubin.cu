// ref_cubin.cu -- TEST INFRASTRUCTURE ONLY.
//
// One translation unit over the reference engine's own kernel sources
// (engine/eos.cu + engine/sph_gravity.cu), included from the reference
// checkout at build time, compiled to a device-only cubin for sm_100 -- "the
// reference's own CUDA build recompiled for sm_100".  oracle/build_oracle.py
// writes it to oracle/_ref/ (never committed); oracle/ref_gpu.py loads it
// with the CUDA driver API and launches its kernels in the order of the
// reference's host launchers, to produce golden stage outputs and the
// reference's GPU step time on the same GB300.
#include "eos.cu"
#include "sph_gravity.cu"
