// Plain-FP64 instantiations of sf_grad_kernel3.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f64(const K3Args &A, int model, bool mp, bool aniso)
{
    if (model == MODEL_HC) {
        if (mp && A.coset)
            return aniso ? dispatch_coset<false, double, MODEL_HC, true, true, true, false, 4, 4, 8, 4>(A)
                         : dispatch_coset<false, double, MODEL_HC, true, false, true, false, 4, 4, 8, 4>(A);
        if (mp) return aniso ? dispatch_k3<false, double, MODEL_HC, true, true, true, false, 4, 8>(A)
                             : dispatch_k3<false, double, MODEL_HC, true, false, true, false, 4, 8>(A);
        if (A.coset)
            return aniso ? dispatch_coset<false, double, MODEL_HC, false, true, true, false, 4, 4, 8, 4>(A)
                         : dispatch_coset<false, double, MODEL_HC, false, false, true, false, 4, 4, 8, 4>(A);
        return aniso ? dispatch_k3<false, double, MODEL_HC, false, true, true, false, 4, 8>(A)
                     : dispatch_k3<false, double, MODEL_HC, false, false, true, false, 4, 8>(A);
    }
    if (model == MODEL_IAM)
        return aniso ? dispatch_k3<false, double, MODEL_IAM, false, true, true, false, 4>(A)
                     : dispatch_k3<false, double, MODEL_IAM, false, false, true, false, 4>(A);
    return aniso ? dispatch_k3<false, double, MODEL_TABLE, false, true, true, false, 4>(A)
                 : dispatch_k3<false, double, MODEL_TABLE, false, false, true, false, 4>(A);
}

}  // namespace dsf
