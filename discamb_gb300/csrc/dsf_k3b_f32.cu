// Batched FP32-bulk instantiations (sf_grad_batch3): many structures of one
// kernel shape in one launch, for the models without the multipole adjoint.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3b_f32(const K3Args &A, int model, bool aniso)
{
    cudaError_t rc;
    if (model == MODEL_HC) {
        if (aniso ? dispatch_pattern<true, float, MODEL_HC, false, true, true, false, kPatD2>(A, rc)
                  : dispatch_pattern<true, float, MODEL_HC, false, false, true, false, kPatD2>(A, rc))
            return rc;
        if (A.coset)
            return aniso ? dispatch_coset<true, float, MODEL_HC, false, true, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A)
                         : dispatch_coset<true, float, MODEL_HC, false, false, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A);
        return aniso ? dispatch_k3<true, float, MODEL_HC, false, true, true, false, 1, 2, 4, 8>(A)
                     : dispatch_k3<true, float, MODEL_HC, false, false, true, false, 1, 2, 4, 8>(A);
    }
    if (model == MODEL_IAM) {
        if (A.inv) {  // operations as n/2 plus their inversion images
            if (aniso && A.coset)
                return dispatch_coset<true, float, MODEL_IAM, false, true, true, true, 2, 2, 4, 4, 8, 8>(A);
            return aniso ? dispatch_k3<true, float, MODEL_IAM, false, true, true, true, 2, 4, 8>(A)
                         : dispatch_k3<true, float, MODEL_IAM, false, false, true, true, 2, 4, 8>(A);
        }
        if (aniso && A.coset) return dispatch_coset<true, float, MODEL_IAM, false, true, true, false, 2, 2, 4, 4, 8, 8>(A);
        return aniso ? dispatch_k3<true, float, MODEL_IAM, false, true, true, false, 2, 4, 8>(A)
                     : dispatch_k3<true, float, MODEL_IAM, false, false, true, false, 2, 4, 8>(A);
    }
    if (A.inv) {  // operations as n/2 plus their inversion images
        // 2/m in the order [1, 2, -1, m]: the Walsh-Hadamard coset kernels, both ADP kinds
        if (aniso ? dispatch_pattern<true, float, MODEL_TABLE, false, true, true, true, kPatC2hB>(A, rc)
                  : dispatch_pattern<true, float, MODEL_TABLE, false, false, true, true, kPatC2hB>(A, rc))
            return rc;
        if (aniso && A.coset) return dispatch_coset<true, float, MODEL_TABLE, false, true, true, true, 2, 2, 4, 4, 8, 8>(A);
        return aniso ? dispatch_k3<true, float, MODEL_TABLE, false, true, true, true, 2, 4, 8>(A)
                     : dispatch_k3<true, float, MODEL_TABLE, false, false, true, true, 2, 4, 8>(A);
    }
    if (aniso && A.coset) return dispatch_coset<true, float, MODEL_TABLE, false, true, true, false, 2, 2, 4, 4, 8, 8>(A);
    return aniso ? dispatch_k3<true, float, MODEL_TABLE, false, true, true, false, 2, 4, 8>(A)
                 : dispatch_k3<true, float, MODEL_TABLE, false, false, true, false, 2, 4, 8>(A);
}

}  // namespace dsf
