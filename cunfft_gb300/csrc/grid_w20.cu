// grid_w20.cu -- gridding kernels for 2m+2 = 20 taps per dimension (m = 9).
#define CG_W 20
#include "grid_inst.inc"
