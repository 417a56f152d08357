// Matvec kernels, ArithSplit instances.
#define ARITH ArithSplit
#define LAUNCH_FN launch_segment_split
#define SMEM_FN segment_smem_split
#define CONFIG_FN configure_kernels_split
#define BATCH_FN launch_batched_split
#define FUSED_FN launch_fused_split
#define PATCH_FN launch_patches_split
#define PATCH_SMEM_FN patch_smem_split
#include "afm_mv_launch.inl"
