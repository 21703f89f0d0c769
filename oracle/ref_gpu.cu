// ref_gpu.cu -- test infrastructure, never part of the library.
//
// The reference's own CUDA time step: usnistgov/phasefield-precipitate-aging
// src/parabola625.cu, src/nucleation.cu and src/discretization.cu, compiled
// where they lie (-I <reference>/src) into one device module by
// `make ref-gpu` (oracle/_ref/ref_step.cubin).  One translation unit stands
// in for the reference's separate compilation of the three files.
// tests/golden/make_ref_gpu_golden.py loads the module with the CUDA driver
// API and launches its kernels in the reference's order to write golden
// steps; nothing else loads it.
#include "parabola625.cu"
#include "nucleation.cu"
#include "discretization.cu"
