// grid_w26.cu -- gridding kernels for 2m+2 = 26 taps per dimension (m = 12).
#define CG_W 26
#include "grid_inst.inc"
