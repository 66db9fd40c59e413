// grid_w14.cu -- gridding kernels for 2m+2 = 14 taps per dimension (m = 6).
#define CG_W 14
#include "grid_inst.inc"
