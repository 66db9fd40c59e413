// grid_w10.cu -- gridding kernels for 2m+2 = 10 taps per dimension (m = 4).
#define CG_W 10
#include "grid_inst.inc"
