// grid_w16.cu -- gridding kernels for 2m+2 = 16 taps per dimension (m = 7).
#define CG_W 16
#include "grid_inst.inc"
