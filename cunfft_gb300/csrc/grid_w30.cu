// grid_w30.cu -- gridding kernels for 2m+2 = 30 taps per dimension (m = 14).
#define CG_W 30
#include "grid_inst.inc"
