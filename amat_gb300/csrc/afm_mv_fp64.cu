// Matvec kernels, ArithF64 instances.
#define ARITH ArithF64
#define LAUNCH_FN launch_segment_fp64
#define SMEM_FN segment_smem_fp64
#define CONFIG_FN configure_kernels_fp64
#define BATCH_FN launch_batched_fp64
#define PATCH_FN launch_patches_fp64
#define PATCH_SMEM_FN patch_smem_fp64
#include "afm_mv_launch.inl"
