// krylov32.cu - the integrator kernels of the Krylov path with FP32 preconditioner factors
// (the ILUT and its triangular solves in FP32; residuals, J v products, GMRES and step control
// in FP64), a module of its own for a parallel build.
#define GB_KERNELS_KRYLOV 32
#include "kernels.cu"
