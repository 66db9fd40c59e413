// grid_w28.cu -- gridding kernels for 2m+2 = 28 taps per dimension (m = 13).
#define CG_W 28
#include "grid_inst.inc"
