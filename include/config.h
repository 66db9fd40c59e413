/*
 * config.h -- build configuration seen by programs written against CUNFFT.
 *
 * The reference bakes these into its ABI at configure time (src/config.h.in,
 * src/config.h:6-49).  This library keeps the committed reference
 * configuration as the ABI of the drop-in plan API: double precision, ptrdiff_t
 * indices, fast Gaussian gridding, cut-off m = 6.  Other cut-offs and FP32 are
 * runtime parameters of the extension API (cunfft_x.h).  The thread-dimension
 * macros are informational (the GB300 kernels choose their own launch shapes);
 * drivers print them in their logs.
 */
#ifndef CONFIG_H
#define CONFIG_H

#define COM_FG_PSI
#define CUNFFT_DOUBLE_PRECISION
#define LARGE_INPUT
#define MILLI_SEC

#ifndef CUT_OFF
#define CUT_OFF 6
#endif

#define THREAD_DIM_X 256
#define THREAD_DIM_Y 256
#define THREAD_DIM 512
#define MAX_NUM_THREADS 1024
#define MAX_BLOCK_DIM_X 1024
#define MAX_BLOCK_DIM_Y 1024
#define MAX_BLOCK_DIM_Z 64
#define MAX_GRID_DIM_X 2147483647
#define MAX_GRID_DIM_Y 65535
#define MAX_GRID_DIM_Z 65535

#endif /* CONFIG_H */
