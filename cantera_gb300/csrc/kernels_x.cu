// kernels_x.cu - the rates, right-hand-side and integrator kernels instantiated for
// mechanisms with the less common rate forms (PLOG, Chebyshev, SRI, Tsang, chemically
// activated falloff).  A module of its own: the out-of-line rate code these need would
// otherwise change the register allocation of the common instantiations in kernels.cu.
#define GB_KERNELS_EXTRA 1
#include "kernels.cu"
