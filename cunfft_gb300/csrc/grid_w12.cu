// grid_w12.cu -- gridding kernels for 2m+2 = 12 taps per dimension (m = 5).
#define CG_W 12
#include "grid_inst.inc"
