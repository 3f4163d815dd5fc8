// FP32-bulk Hansen-Coppens instantiations of sf_grad_kernel3 with the
// multipole-parameter adjoint (own translation unit: the largest kernels).
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f32_hc_mp(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool aniso,
                                int n_tiles, int n_chunks, size_t smem, cudaStream_t st)
{
    if (L.coset)
        return aniso ? dispatch_coset<float, true, true, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st)
                     : dispatch_coset<float, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st);
    return aniso ? dispatch_k3<float, MODEL_HC, true, true, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st)
                 : dispatch_k3<float, MODEL_HC, true, false, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st);
}

}  // namespace dsf
