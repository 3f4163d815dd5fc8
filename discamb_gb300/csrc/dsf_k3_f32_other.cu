// FP32-bulk IAM and tabulated-form-factor instantiations of sf_grad_kernel3.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f32_other(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool aniso,
                                int n_tiles, int n_chunks, size_t smem, cudaStream_t st)
{
    if (S.model == MODEL_IAM)
        return aniso ? dispatch_k3<float, MODEL_IAM, false, true, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st)
                     : dispatch_k3<float, MODEL_IAM, false, false, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st);
    return aniso ? dispatch_k3<float, MODEL_TABLE, false, true, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st)
                 : dispatch_k3<float, MODEL_TABLE, false, false, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st);
}

}  // namespace dsf
