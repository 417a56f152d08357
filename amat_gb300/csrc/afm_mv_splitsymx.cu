// Matvec kernels, ArithSplitSymX instances (FP64 vectors, double-float
// products from the corrected symmetric arena: the inner product of the
// FP64-vector mixed-precision solve).
#define ARITH ArithSplitSymX
#define LAUNCH_FN launch_segment_splitsymx
#define SMEM_FN segment_smem_splitsymx
#define CONFIG_FN configure_kernels_splitsymx
#define PATCH_FN launch_patches_splitsymx
#define PATCH_SMEM_FN patch_smem_splitsymx
#include "afm_mv_launch.inl"
