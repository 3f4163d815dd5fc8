// Structure-factor-only FP32 kernels of the HC model (sf_grad_kernel3 with
// GRAD = false): the reference's calculateStructureFactors runs its engine
// with every derivative switched off (HansenCoppensStructureFactorCalculator
// .cpp:305-326); here the adjoint is compiled out.  The same operation counts
// and coset pairs as dsf_k3_f32_hc.cu.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3f_hc(const K3Args &A, bool aniso)
{
    cudaError_t rc;
    if (aniso ? dispatch_pattern<false, float, MODEL_HC, false, true, false, false, kPatD2>(A, rc)
              : dispatch_pattern<false, float, MODEL_HC, false, false, false, false, kPatD2>(A, rc))
        return rc;
    if (A.coset)
        return aniso ? dispatch_coset<false, float, MODEL_HC, false, true, false, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A)
                     : dispatch_coset<false, float, MODEL_HC, false, false, false, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A);
    return aniso ? dispatch_k3<false, float, MODEL_HC, false, true, false, false, 2, 4, 8>(A)
                 : dispatch_k3<false, float, MODEL_HC, false, false, false, false, 2, 4, 8>(A);
}

}  // namespace dsf
