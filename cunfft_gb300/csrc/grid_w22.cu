// grid_w22.cu -- gridding kernels for 2m+2 = 22 taps per dimension (m = 10).
#define CG_W 22
#include "grid_inst.inc"
