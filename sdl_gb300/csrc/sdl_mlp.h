// Launchers of the learned tracklet pre-filter's kernels (sdl_mlp.cu).
#pragma once
#include <cuda_runtime.h>

#include "sdl_mlp.cuh"

namespace sdlg {

// FP32 parameters (kMlpParams) -> packed inference weights (kPackBytes) with threshold thr
void launch_mlp_pack(const float* params, unsigned char* pack, float thr, cudaStream_t s);
// logits of n feature rows on the tensor cores; *status |= 1 if a wait gave up
void launch_mlp_score(const float* x, int64_t n, const unsigned char* pack, float* logits, unsigned int* status, int n_sm,
                      cudaStream_t s);
// one training step's forward + backward (see k_mlp_fwd_bwd)
cudaError_t launch_mlp_fwd_bwd(const float* X, const float* Y, const float* W, const int32_t* order, int64_t start,
                               int64_t count, float pos_weight, float inv_norm, const float* params, float* grad,
                               double* loss, cudaStream_t s);
// Adam update with bias corrections c1 = 1 - beta1^t, c2 = 1 - beta2^t
void launch_mlp_adam(float* p, float* g, float* m, float* v, float lr, float c1, float c2, cudaStream_t s);
size_t mlp_train_smem();

}  // namespace sdlg
