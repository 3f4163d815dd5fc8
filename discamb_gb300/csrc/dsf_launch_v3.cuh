// Launch helpers of sf_grad_kernel3: one instantiation per (precision, model,
// multipole adjoint, ADP kind, symmetry-operation count); counts other than the
// compiled ones use the runtime loop.  The instantiations are spread over
// three translation units so they compile in parallel.
#pragma once
#include "dsf_sf_kernel.cuh"

namespace dsf {

template <typename R, int MODEL, bool MP, bool ANISO, int NSC>
cudaError_t launch_k3(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles, int n_chunks,
                      size_t smem, cudaStream_t st)
{
    auto k = sf_grad_kernel3<R, MODEL, MP, ANISO, NSC>;
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

cudaError_t launch_k3_f32_hc(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool mp, bool aniso,
                             int n_tiles, int n_chunks, size_t smem, cudaStream_t st);
cudaError_t launch_k3_f32_other(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool aniso,
                                int n_tiles, int n_chunks, size_t smem, cudaStream_t st);
cudaError_t launch_k3_f64(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool mp, bool aniso,
                          int n_tiles, int n_chunks, size_t smem, cudaStream_t st);

}  // namespace dsf
