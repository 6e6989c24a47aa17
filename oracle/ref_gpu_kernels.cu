// Reference GPU kernels, compiled from the reference sources for sm_103a --
// TEST INFRASTRUCTURE ONLY.
//
// `make -C oracle refgpu` compiles this file (which only includes the
// reference headers where they lie, through the per-block-size overlay of
// `make ref`) into oracle/_ref/ref_kernels_bs<N>.cubin, and lists the
// kernels' symbol names (from the host object of the same file) in
// oracle/_ref/ref_kernels_bs<N>.names.  oracle/ref_gpu_harness.cpp loads the
// cubin with the driver API so tests/golden/make_golden_gpu.py can record
// the reference kernels' outputs as golden vectors and time them on GB300.
#include "common.h"
#include "isai_bsr.h"
#include "bcsc2bcsr.h"
#include "bcsc2bcsrAndSpMV.h"

template __global__ void reorder_bcsc_val_to_bcsr_bs5<double>(int, const int*, const double*,
                                                               double*);
