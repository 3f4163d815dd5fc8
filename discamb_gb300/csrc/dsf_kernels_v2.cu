// Instantiations and launch of the table-streaming structure-factor kernel
// (dsf_sf_kernel.cuh).  FP32-bulk: symmetry-operation counts 2, 4, 8 compiled
// with the operation loop unrolled, other counts with a runtime loop; plain
// FP64: runtime loop.
#include "dsf_sf_kernel.cuh"

namespace dsf {

template <typename R, bool MP, bool ANISO, int NSC>
static cudaError_t launch_one(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles,
                              int n_chunks, size_t smem, cudaStream_t st)
{
    auto k = sf_grad_kernel2<R, MP, ANISO, NSC>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<dim3(n_tiles, n_chunks), kTileAtoms, smem, st>>>(S, C, L);
    return cudaGetLastError();
}

template <typename R, bool MP, bool ANISO>
static cudaError_t dispatch_ns(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, int n_tiles,
                               int n_chunks, size_t smem, cudaStream_t st)
{
    if constexpr (sizeof(R) == 4) {
        switch (S.n_sym) {
        case 2: return launch_one<R, MP, ANISO, 2>(S, C, L, n_tiles, n_chunks, smem, st);
        case 4: return launch_one<R, MP, ANISO, 4>(S, C, L, n_tiles, n_chunks, smem, st);
        case 8: return launch_one<R, MP, ANISO, 8>(S, C, L, n_tiles, n_chunks, smem, st);
        default: break;
        }
    }
    return launch_one<R, MP, ANISO, 0>(S, C, L, n_tiles, n_chunks, smem, st);
}

size_t sf2_smem_bytes(bool fp64, bool mp, int ht, int n_sym, int max_types)
{
    if (fp64) return mp ? sf_smem_bytes<double, true>(ht, n_sym, max_types) : sf_smem_bytes<double, false>(ht, n_sym, max_types);
    return mp ? sf_smem_bytes<float, true>(ht, n_sym, max_types) : sf_smem_bytes<float, false>(ht, n_sym, max_types);
}

cudaError_t launch_sf2(const DevStructure &S, const CallBuffers &C, const SfLaunch &L, bool fp64, bool mp, bool aniso,
                       int n_tiles, int n_chunks, cudaStream_t st)
{
    const size_t smem = sf2_smem_bytes(fp64, mp, L.ht, S.n_sym, L.max_types);
    if (fp64) {
        if (mp) return aniso ? dispatch_ns<double, true, true>(S, C, L, n_tiles, n_chunks, smem, st)
                             : dispatch_ns<double, true, false>(S, C, L, n_tiles, n_chunks, smem, st);
        return aniso ? dispatch_ns<double, false, true>(S, C, L, n_tiles, n_chunks, smem, st)
                     : dispatch_ns<double, false, false>(S, C, L, n_tiles, n_chunks, smem, st);
    }
    if (mp) return aniso ? dispatch_ns<float, true, true>(S, C, L, n_tiles, n_chunks, smem, st)
                         : dispatch_ns<float, true, false>(S, C, L, n_tiles, n_chunks, smem, st);
    return aniso ? dispatch_ns<float, false, true>(S, C, L, n_tiles, n_chunks, smem, st)
                 : dispatch_ns<float, false, false>(S, C, L, n_tiles, n_chunks, smem, st);
}

}  // namespace dsf
