// FP32-bulk Hansen-Coppens instantiations of sf_grad_kernel3 without the
// multipole adjoint, and the launch entry.
#include "dsf_launch_v3.cuh"

namespace dsf {

cudaError_t launch_k3_f32_hc(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool mp, bool aniso,
                             int n_tiles, int n_chunks, size_t smem, cudaStream_t st)
{
    if (mp) return launch_k3_f32_hc_mp(S, C, L, aniso, n_tiles, n_chunks, smem, st);
    if (L.coset)
        return aniso ? dispatch_coset<float, false, true, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st)
                     : dispatch_coset<float, false, false, 2, 2, 4, 4, 4, 2, 8, 8, 8, 4>(S, C, L, n_tiles, n_chunks, smem, st);
    return aniso ? dispatch_k3<float, MODEL_HC, false, true, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st)
                 : dispatch_k3<float, MODEL_HC, false, false, 2, 4, 8>(S, C, L, n_tiles, n_chunks, smem, st);
}

size_t sf3_smem_bytes(bool fp64, bool mp, int ht, int n_sym, int max_types)
{
    if (fp64) return mp ? sf_smem_bytes<double, true>(ht, n_sym, max_types) : sf_smem_bytes<double, false>(ht, n_sym, max_types);
    return mp ? sf_smem_bytes<float, true>(ht, n_sym, max_types) : sf_smem_bytes<float, false>(ht, n_sym, max_types);
}

cudaError_t launch_sf3(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool fp64, bool mp, bool aniso,
                       int n_tiles, int n_chunks, cudaStream_t st)
{
    const bool mp_hc = mp && S.model == MODEL_HC;
    const size_t smem = sf3_smem_bytes(fp64, mp_hc, L.ht, S.n_sym, L.max_types);
    if (fp64) return launch_k3_f64(S, C, L, mp_hc, aniso, n_tiles, n_chunks, smem, st);
    if (S.model == MODEL_HC) return launch_k3_f32_hc(S, C, L, mp_hc, aniso, n_tiles, n_chunks, smem, st);
    return launch_k3_f32_other(S, C, L, aniso, n_tiles, n_chunks, smem, st);
}

}  // namespace dsf
