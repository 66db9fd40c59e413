// grid_w8.cu -- gridding kernels for 2m+2 = 8 taps per dimension (m = 3).
#define CG_W 8
#include "grid_inst.inc"
