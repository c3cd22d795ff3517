// ORACLE -- test infrastructure, not product code.
//
// Translation unit that compiles the reference DiskDyn kernels, unmodified, into a cubin
// for sm_103a.  The reference sources are read in place through the include path given
// by build_ref.py (its src/ directory); nothing of them is copied here.  The
// __constant__ / __device__ symbols that the reference defines in ddyn.cu (lines 29-33) are
// defined here with the same names and sizes, because ddyn.cu also holds main().
#include <stdio.h>
#include "ddyn.cuh"
__constant__ double size[nsize];
__constant__ float  beta[nsize];
__constant__ float  betasw[nsize];
__constant__ float  q[nsize];
__device__   double doubletmp;
#include "gpu_functions.cu"
