// Structure-factor-only FP32 kernels of the IAM and tabulated models
// (sf_grad_kernel3 with GRAD = false; AnyScattererStructureFactorCalculator::
// calculateStructureFactors, src/Scattering/AnyScattererStructureFactor
// Calculator.cpp:293-433, evaluates F without the derivative loop).  The same
// operation counts and coset pairs as dsf_k3_f32_other.cu.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3f_other(const K3Args &A, int model, bool aniso)
{
    if (model == MODEL_IAM) {
        if (A.inv) {  // operations as n/2 plus their inversion images
            if (aniso && A.coset)
                return dispatch_coset<false, float, MODEL_IAM, false, true, false, true, 2, 2, 4, 4, 8, 8>(A);
            return aniso ? dispatch_k3<false, float, MODEL_IAM, false, true, false, true, 2, 4, 8>(A)
                         : dispatch_k3<false, float, MODEL_IAM, false, false, false, true, 2, 4, 8>(A);
        }
        if (aniso && A.coset) return dispatch_coset<false, float, MODEL_IAM, false, true, false, false, 2, 2, 4, 4, 8, 8>(A);
        return aniso ? dispatch_k3<false, float, MODEL_IAM, false, true, false, false, 2, 4, 8>(A)
                     : dispatch_k3<false, float, MODEL_IAM, false, false, false, false, 2, 4, 8>(A);
    }
    if (A.inv) {  // operations as n/2 plus their inversion images
        if (aniso && A.coset) return dispatch_coset<false, float, MODEL_TABLE, false, true, false, true, 2, 2, 4, 4, 8, 8>(A);
        return aniso ? dispatch_k3<false, float, MODEL_TABLE, false, true, false, true, 2, 4, 8>(A)
                     : dispatch_k3<false, float, MODEL_TABLE, false, false, false, true, 2, 4, 8>(A);
    }
    if (aniso && A.coset) return dispatch_coset<false, float, MODEL_TABLE, false, true, false, false, 2, 2, 4, 4, 8, 8>(A);
    return aniso ? dispatch_k3<false, float, MODEL_TABLE, false, true, false, false, 2, 4, 8>(A)
                 : dispatch_k3<false, float, MODEL_TABLE, false, false, false, false, 2, 4, 8>(A);
}

}  // namespace dsf
