// grid_w18.cu -- gridding kernels for 2m+2 = 18 taps per dimension (m = 8).
#define CG_W 18
#include "grid_inst.inc"
