// Matvec kernels, ArithF32 instances.
#define ARITH ArithF32
#define LAUNCH_FN launch_segment_fp32
#define SMEM_FN segment_smem_fp32
#define CONFIG_FN configure_kernels_fp32
#define BATCH_FN launch_batched_fp32
#define PATCH_FN launch_patches_fp32
#define PATCH_SMEM_FN patch_smem_fp32
#include "afm_mv_launch.inl"
