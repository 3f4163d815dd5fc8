// FP32-bulk Hansen-Coppens instantiations of sf_grad_kernel3 without the
// multipole adjoint, and the launch entry of the single-structure kernels.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f32_hc(const K3Args &A, bool mp, bool aniso)
{
    if (mp) return launch_k3_f32_hc_mp(A, aniso);
    cudaError_t rc;
    if (aniso ? dispatch_pattern<false, float, MODEL_HC, false, true, true, false, kPatD2>(A, rc)
              : dispatch_pattern<false, float, MODEL_HC, false, false, true, false, kPatD2>(A, rc))
        return rc;
    if (A.coset)
        return aniso ? dispatch_coset<false, float, MODEL_HC, false, true, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A)
                     : dispatch_coset<false, float, MODEL_HC, false, false, true, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(A);
    return aniso ? dispatch_k3<false, float, MODEL_HC, false, true, true, false, 2, 4, 8>(A)
                 : dispatch_k3<false, float, MODEL_HC, false, false, true, false, 2, 4, 8>(A);
}

size_t sf3_smem_bytes(bool fp64, bool mp, int ht, int n_sym, int max_types, bool table)
{
    if (fp64) return mp ? sf_smem_bytes<double, true>(ht, n_sym, max_types) : sf_smem_bytes<double, false>(ht, n_sym, max_types);
    return mp ? sf_smem_bytes<float, true>(ht, n_sym, max_types)
              : sf_smem_bytes<float, false>(ht, n_sym, max_types, table && !table_count_compiled(n_sym));
}

cudaError_t launch_sf3(const K3Args &A, int model, bool fp64, bool mp, bool aniso)
{
    const bool mp_hc = mp && model == MODEL_HC;
    if (fp64) return launch_k3_f64(A, model, mp_hc, aniso);
    if (!A.grad && !mp_hc) return model == MODEL_HC ? launch_k3f_hc(A, aniso) : launch_k3f_other(A, model, aniso);
    if (model == MODEL_HC) return launch_k3_f32_hc(A, mp_hc, aniso);
    return launch_k3_f32_other(A, model, aniso);
}

}  // namespace dsf
