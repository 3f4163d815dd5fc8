// Plain-FP64 instantiations of sf_grad_kernel3.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f64(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool mp, bool aniso,
                          int n_tiles, int n_chunks, size_t smem, cudaStream_t st)
{
    if (S.model == MODEL_HC) {
        if (mp && L.coset)
            return aniso ? dispatch_coset<double, true, true, 4, 4, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st)
                         : dispatch_coset<double, true, false, 4, 4, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st);
        if (mp) return aniso ? dispatch_k3<double, MODEL_HC, true, true, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st)
                             : dispatch_k3<double, MODEL_HC, true, false, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st);
        if (L.coset)
            return aniso ? dispatch_coset<double, false, true, 4, 4, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st)
                         : dispatch_coset<double, false, false, 4, 4, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st);
        return aniso ? dispatch_k3<double, MODEL_HC, false, true, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st)
                     : dispatch_k3<double, MODEL_HC, false, false, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st);
    }
    if (S.model == MODEL_IAM)
        return aniso ? dispatch_k3<double, MODEL_IAM, false, true>(S, C, L, n_tiles, n_chunks, smem, st)
                     : dispatch_k3<double, MODEL_IAM, false, false>(S, C, L, n_tiles, n_chunks, smem, st);
    return aniso ? dispatch_k3<double, MODEL_TABLE, false, true>(S, C, L, n_tiles, n_chunks, smem, st)
                 : dispatch_k3<double, MODEL_TABLE, false, false>(S, C, L, n_tiles, n_chunks, smem, st);
}

}  // namespace dsf
