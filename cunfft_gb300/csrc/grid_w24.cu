// grid_w24.cu -- gridding kernels for 2m+2 = 24 taps per dimension (m = 11).
#define CG_W 24
#include "grid_inst.inc"
