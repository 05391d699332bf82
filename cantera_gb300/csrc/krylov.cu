// krylov.cu - the integrator kernels of the Krylov path (the mole reactor with GMRES and the
// adaptive preconditioner) with FP64 preconditioner factors, and the batched incomplete
// factorisation, instantiated in a module of their own so that they compile in parallel with
// the others and leave the dense integrator's register allocation untouched.
#define GB_KERNELS_KRYLOV 64
#include "kernels.cu"
