// grid_w4.cu -- gridding kernels for 2m+2 = 4 taps per dimension (m = 1).
#define CG_W 4
#include "grid_inst.inc"
