// grid_w32.cu -- gridding kernels for 2m+2 = 32 taps per dimension (m = 15).
#define CG_W 32
#include "grid_inst.inc"
