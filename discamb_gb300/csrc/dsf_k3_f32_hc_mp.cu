// FP32-bulk Hansen-Coppens instantiations of sf_grad_kernel3 with the
// multipole-parameter adjoint (own translation unit: the largest kernels).
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f32_hc_mp(const K3Args &A, bool aniso)
{
    cudaError_t rc;
    if (aniso ? dispatch_pattern<false, float, MODEL_HC, true, true, true, false, kPatD2>(A, rc)
              : dispatch_pattern<false, float, MODEL_HC, true, false, true, false, kPatD2>(A, rc))
        return rc;
    if (A.coset)
        return aniso ? dispatch_coset<false, float, MODEL_HC, true, true, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A)
                     : dispatch_coset<false, float, MODEL_HC, true, false, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A);
    return aniso ? dispatch_k3<false, float, MODEL_HC, true, true, true, false, 2, 4, 8>(A)
                 : dispatch_k3<false, float, MODEL_HC, true, false, true, false, 2, 4, 8>(A);
}

}  // namespace dsf
