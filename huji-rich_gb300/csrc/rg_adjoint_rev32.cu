// rg_adjoint_rev32.cu -- the FP32 build of the face and cell reverse kernels
// (rg_adjoint_rev.cu) for the FP32-mixed adjoint: the reverse of the
// reconstruction, the limiter and Hllc in FP32, as the FP32-mixed step
// computes them forward; the transposed extensive gather, the transposed
// cell update and every stored adjoint stay FP64, as the step keeps its
// extensive accumulation and energy conversion in FP64.
#define RG_ADJ_REAL float
#define RG_ADJ_FP64 0
#include "rg_adjoint_rev.cu"
