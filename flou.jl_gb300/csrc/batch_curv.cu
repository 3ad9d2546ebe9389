// The batched-stage kernels for instances on general geometry (batch_kernels.cuh): the same
// operators as batch.cu's list, with the CURV tiles and face nodes.
#include "batch_kernels.cuh"
namespace flou {
const BatchKernel kBatchKernelsCurv[] = {
    {2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 128, true,
     batch_stage_kernel<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 128, true>,
     batch_smem_bytes<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 128, true>()},
    {2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 256, true,
     batch_stage_kernel<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 256, true>,
     batch_smem_bytes<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 256, true>()},
    {3, FLOU_EQ_EULER, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, 512, true,
     batch_stage_kernel<3, FLOU_EQ_EULER, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, 512, true>,
     batch_smem_bytes<3, FLOU_EQ_EULER, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, 512, true>()},
};
const int kNumBatchKernelsCurv = sizeof(kBatchKernelsCurv) / sizeof(kBatchKernelsCurv[0]);
}  // namespace flou
