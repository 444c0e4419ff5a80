// The FP64 instantiation of the batched solver kernel (k_nasoq_batch<double>,
// launch_batch<double>, batch_prepare<double>) in a translation unit of its
// own, so that it compiles in parallel with the FP32 one: batch.cu with
// NQG_BATCH_FP64_UNIT defined, which keeps only its templates and this
// instantiation.
#define NQG_BATCH_FP64_UNIT
#include "batch.cu"
