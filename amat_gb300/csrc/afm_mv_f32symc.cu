// Matvec kernels, ArithF32SymC instances (the corrected symmetric arena, u in
// FP32, element rows summed in FP32 and into v in FP64: the inner product of
// symmetric inner format 5).
#define ARITH ArithF32SymC
#define LAUNCH_FN launch_segment_f32symc
#define SMEM_FN segment_smem_f32symc
#define CONFIG_FN configure_kernels_f32symc
#define PATCH_FN launch_patches_f32symc
#define PATCH_SMEM_FN patch_smem_f32symc
#include "afm_mv_launch.inl"
