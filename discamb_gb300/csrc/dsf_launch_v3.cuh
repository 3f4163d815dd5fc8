// Launch helpers of sf_grad_kernel3: one instantiation per (precision, model,
// multipole adjoint, ADP kind, symmetry-operation count); counts other than the
// compiled ones use the runtime loop.  The instantiations are spread over
// three translation units so they compile in parallel.
#pragma once
#include "dsf_sf_kernel.cuh"

namespace dsf {

template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS = 0>
cudaError_t launch_k3(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles, int n_chunks,
                      size_t smem, cudaStream_t st)
{
    auto k = sf_grad_kernel3<R, MODEL, MP, ANISO, NSC, CS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<dim3(n_tiles, n_chunks), kTileAtoms, smem, st>>>(S, C, L);
    return cudaGetLastError();
}

// compiled operation counts first, runtime count last
template <typename R, int MODEL, bool MP, bool ANISO>
cudaError_t dispatch_k3(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles, int n_chunks,
                        size_t smem, cudaStream_t st)
{
    return launch_k3<R, MODEL, MP, ANISO, 0>(S, C, L, n_tiles, n_chunks, smem, st);
}

template <typename R, int MODEL, bool MP, bool ANISO, int N0, int... NS>
cudaError_t dispatch_k3(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles, int n_chunks,
                        size_t smem, cudaStream_t st)
{
    if (S.n_sym == N0) return launch_k3<R, MODEL, MP, ANISO, N0>(S, C, L, n_tiles, n_chunks, smem, st);
    return dispatch_k3<R, MODEL, MP, ANISO, NS...>(S, C, L, n_tiles, n_chunks, smem, st);
}

// HC, operations in sign-diagonal cosets: the class-sum kernels of the
// compiled (operation count, coset size) pairs; the engine sets L.coset only
// for those pairs (coset_form_compiled)
template <typename R, bool MP, bool ANISO>
cudaError_t dispatch_coset(const DevStructure &, const CallBuffers &, const SfLaunch &, int, int, size_t, cudaStream_t)
{
    return cudaErrorInvalidValue;
}

template <typename R, bool MP, bool ANISO, int N0, int CS0, int... NC>
cudaError_t dispatch_coset(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles, int n_chunks,
                           size_t smem, cudaStream_t st)
{
    if (S.n_sym == N0 && L.coset == CS0)
        return launch_k3<R, MODEL_HC, MP, ANISO, N0, CS0>(S, C, L, n_tiles, n_chunks, smem, st);
    return dispatch_coset<R, MP, ANISO, NC...>(S, C, L, n_tiles, n_chunks, smem, st);
}

// (operation count, coset size) pairs with compiled class-sum kernels
__host__ inline bool coset_form_compiled(bool fp64, int n_sym, int cs)
{
    if (fp64) return (n_sym == 4 && cs == 4) || (n_sym == 8 && cs == 4);
    return (n_sym == 2 && cs == 2) || (n_sym == 4 && (cs == 4 || cs == 2)) || (n_sym == 8 && (cs == 8 || cs == 4));
}

cudaError_t launch_k3_f32_hc(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool mp, bool aniso,
                             int n_tiles, int n_chunks, size_t smem, cudaStream_t st);
cudaError_t launch_k3_f32_hc_mp(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool aniso,
                                int n_tiles, int n_chunks, size_t smem, cudaStream_t st);
cudaError_t launch_k3_f32_other(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool aniso,
                                int n_tiles, int n_chunks, size_t smem, cudaStream_t st);
cudaError_t launch_k3_f64(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool mp, bool aniso,
                          int n_tiles, int n_chunks, size_t smem, cudaStream_t st);

}  // namespace dsf
