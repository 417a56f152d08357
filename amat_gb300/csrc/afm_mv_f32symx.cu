// Matvec kernels, ArithF32SymX instances (FP32 products from the symmetric
// inner arena with its BF16 correction plane, double-float accumulation).
#define ARITH ArithF32SymX
#define LAUNCH_FN launch_segment_f32symx
#define SMEM_FN segment_smem_f32symx
#define CONFIG_FN configure_kernels_f32symx
#define PATCH_FN launch_patches_f32symx
#define PATCH_SMEM_FN patch_smem_f32symx
#include "afm_mv_launch.inl"
