// Matvec kernels, ArithSplit instances.
#define ARITH ArithSplit
#define LAUNCH_FN launch_segment_split
#define SMEM_FN segment_smem_split
#include "afm_mv_launch.inl"
