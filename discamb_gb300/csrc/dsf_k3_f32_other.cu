// FP32-bulk IAM and tabulated-form-factor instantiations of sf_grad_kernel3.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f32_other(const K3Args &A, int model, bool aniso)
{
    if (model == MODEL_IAM) {
        if (A.inv) {  // operations as n/2 plus their inversion images
            if (aniso && A.coset)
                return dispatch_coset<false, float, MODEL_IAM, false, true, true, true, 2, 2, 4, 4, 8, 8>(A);
            return aniso ? dispatch_k3<false, float, MODEL_IAM, false, true, true, true, 2, 4, 8>(A)
                         : dispatch_k3<false, float, MODEL_IAM, false, false, true, true, 2, 4, 8>(A);
        }
        if (aniso && A.coset) return dispatch_coset<false, float, MODEL_IAM, false, true, true, false, 2, 2, 4, 4, 8, 8>(A);
        return aniso ? dispatch_k3<false, float, MODEL_IAM, false, true, true, false, 2, 4, 8>(A)
                     : dispatch_k3<false, float, MODEL_IAM, false, false, true, false, 2, 4, 8>(A);
    }
    if (A.inv) {  // operations as n/2 plus their inversion images
        cudaError_t rc;  // 2/m in the order [1, 2, -1, m]: the Walsh-Hadamard coset kernels, both ADP kinds
        if (aniso ? dispatch_pattern<false, float, MODEL_TABLE, false, true, true, true, kPatC2hB>(A, rc)
                  : dispatch_pattern<false, float, MODEL_TABLE, false, false, true, true, kPatC2hB>(A, rc))
            return rc;
        if (aniso && A.coset) return dispatch_coset<false, float, MODEL_TABLE, false, true, true, true, 2, 2, 4, 4, 8, 8>(A);
        return aniso ? dispatch_k3<false, float, MODEL_TABLE, false, true, true, true, 2, 4, 8>(A)
                     : dispatch_k3<false, float, MODEL_TABLE, false, false, true, true, 2, 4, 8>(A);
    }
    if (aniso && A.coset) return dispatch_coset<false, float, MODEL_TABLE, false, true, true, false, 2, 2, 4, 4, 8, 8>(A);
    return aniso ? dispatch_k3<false, float, MODEL_TABLE, false, true, true, false, 2, 4, 8>(A)
                 : dispatch_k3<false, float, MODEL_TABLE, false, false, true, false, 2, 4, 8>(A);
}

}  // namespace dsf
