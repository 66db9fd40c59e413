// grid_w6.cu -- gridding kernels for 2m+2 = 6 taps per dimension (m = 2).
#define CG_W 6
#include "grid_inst.inc"
