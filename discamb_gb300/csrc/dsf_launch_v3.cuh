// Launch helpers of sf_grad_kernel3 / sf_grad_batch3: one instantiation per
// (precision, model, multipole adjoint, ADP kind, symmetry-operation count,
// coset size); counts other than the compiled ones use the runtime loop.  The
// instantiations are spread over several translation units so they compile in
// parallel; the batched form exists for the FP32 kernels without the multipole
// adjoint (dsf_k3b_f32.cu).
#pragma once
#include "dsf_sf_kernel.cuh"

namespace dsf {

// everything a launch needs: one structure (S, C, L, grid n_tiles x n_chunks)
// or a batch (B, grid of `blocks`)
struct K3Args {
    const DevStructure *S = nullptr;
    const CallBuffers *C = nullptr;
    const SfLaunch *L = nullptr;
    const SignTable *G = nullptr;
    const SfBatch *B = nullptr;
    int n_sym = 0, coset = 0;
    bool grad = true;  // false: structure factors only (single-structure FP32 kernels without the adjoint)
    bool inv = false;  // operations as n/2 plus their images under an inversion at the origin (generic models)
    int pattern = 0;   // cosets of four in the order of a known sign group (kPatD2, kPatC2hB), else 0
    bool occ3 = false; // the register-capped form (three blocks per SM) where it is compiled (occ3_kernel)
    int n_tiles = 0, n_chunks = 0, blocks = 0;
    size_t smem = 0;
    cudaStream_t st = nullptr;
};

template <typename K, typename... Args>
cudaError_t launch_with(K k, dim3 grid, size_t smem, cudaStream_t st, const Args &...args)
{
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kTileAtoms, smem, st>>>(args...);
    return cudaGetLastError();
}

// kernels with a register-capped form of three blocks per SM: FP32 HC multipole adjoint, sign-group cosets
template <bool BATCH, typename R, int MODEL, bool MP, bool GRAD, int PAT>
constexpr bool occ3_kernel() { return !BATCH && sizeof(R) == 4 && MODEL == MODEL_HC && MP && GRAD && PAT != 0; }

template <bool BATCH, typename R, int MODEL, bool MP, bool ANISO, bool GRAD, bool INV, int NSC, int CS = 0,
          int PAT = 0>
cudaError_t launch_k3(const K3Args &A)
{
    constexpr bool OCC4 = occ4_kernel<R, MODEL, NSC>();
    if constexpr (occ3_kernel<BATCH, R, MODEL, MP, GRAD, PAT>())
        if (A.occ3)
            return launch_with(sf_grad_kernel3_occ3<R, MODEL, MP, ANISO, NSC, CS, true, INV, PAT>,
                               dim3(A.n_tiles, A.n_chunks), A.smem, A.st, *A.S, *A.C, *A.L, *A.G);
    const dim3 grid = BATCH ? dim3(A.blocks) : dim3(A.n_tiles, A.n_chunks);
    static_assert(GRAD || !BATCH, "structure-factor-only kernels: single structures");
    if constexpr (!GRAD && OCC4)
        return launch_with(sf_grad_kernel3_occ4<R, MODEL, MP, ANISO, NSC, CS, false, INV, PAT>, grid, A.smem, A.st,
                           *A.S, *A.C, *A.L, *A.G);
    else if constexpr (!GRAD)
        return launch_with(sf_grad_kernel3<R, MODEL, MP, ANISO, NSC, CS, false, INV, PAT>, grid, A.smem, A.st, *A.S,
                           *A.C, *A.L, *A.G);
    else if constexpr (BATCH && OCC4)
        return launch_with(sf_grad_batch3_occ4<R, MODEL, MP, ANISO, NSC, CS, INV, PAT>, grid, A.smem, A.st, *A.B,
                           *A.G);
    else if constexpr (BATCH)
        return launch_with(sf_grad_batch3<R, MODEL, MP, ANISO, NSC, CS, INV, PAT>, grid, A.smem, A.st, *A.B, *A.G);
    else if constexpr (OCC4)
        return launch_with(sf_grad_kernel3_occ4<R, MODEL, MP, ANISO, NSC, CS, true, INV, PAT>, grid, A.smem, A.st,
                           *A.S, *A.C, *A.L, *A.G);
    else
        return launch_with(sf_grad_kernel3<R, MODEL, MP, ANISO, NSC, CS, true, INV, PAT>, grid, A.smem, A.st, *A.S,
                           *A.C, *A.L, *A.G);
}

// cosets of four in a known sign group's order (A.pattern == PAT): the Walsh-Hadamard kernels of the compiled
// operation counts (4, 8); false when none applies (the caller then takes the general coset kernels)
template <bool BATCH, typename R, int MODEL, bool MP, bool ANISO, bool GRAD, bool INV, int PAT>
bool dispatch_pattern(const K3Args &A, cudaError_t &rc)
{
    if (A.pattern != PAT || A.coset != 4) return false;
    if (A.n_sym == 4) rc = launch_k3<BATCH, R, MODEL, MP, ANISO, GRAD, INV, 4, 4, PAT>(A);
    else if (A.n_sym == 8 && !INV) rc = launch_k3<BATCH, R, MODEL, MP, ANISO, GRAD, INV, 8, 4, PAT>(A);
    else return false;
    return true;
}

// compiled operation counts first, runtime count last (INV kernels exist only for compiled counts: the
// runtime one is never reached with A.inv set, the engine sets it only for those counts)
template <bool BATCH, typename R, int MODEL, bool MP, bool ANISO, bool GRAD, bool INV>
cudaError_t dispatch_k3(const K3Args &A)
{
    if constexpr (INV) return cudaErrorInvalidValue;
    else return launch_k3<BATCH, R, MODEL, MP, ANISO, GRAD, false, 0>(A);
}

template <bool BATCH, typename R, int MODEL, bool MP, bool ANISO, bool GRAD, bool INV, int N0, int... NS>
cudaError_t dispatch_k3(const K3Args &A)
{
    if (A.n_sym == N0) return launch_k3<BATCH, R, MODEL, MP, ANISO, GRAD, INV, N0>(A);
    return dispatch_k3<BATCH, R, MODEL, MP, ANISO, GRAD, INV, NS...>(A);
}

// operations in sign-diagonal cosets: the coset kernels of the compiled
// (operation count, coset size) pairs; the engine sets L.coset only for those
// pairs (coset_form_compiled)
template <bool BATCH, typename R, int MODEL, bool MP, bool ANISO, bool GRAD, bool INV>
cudaError_t dispatch_coset(const K3Args &)
{
    return cudaErrorInvalidValue;
}

template <bool BATCH, typename R, int MODEL, bool MP, bool ANISO, bool GRAD, bool INV, int N0, int CS0, int... NC>
cudaError_t dispatch_coset(const K3Args &A)
{
    if (A.n_sym == N0 && A.coset == CS0) return launch_k3<BATCH, R, MODEL, MP, ANISO, GRAD, INV, N0, CS0>(A);
    return dispatch_coset<BATCH, R, MODEL, MP, ANISO, GRAD, INV, NC...>(A);
}

// (operation count, coset size) pairs with compiled coset kernels.  HC: both
// ADP kinds; IAM and tabulated: the anisotropic kernels, one coset of all
// operations (their launches of isotropic tiles use the general form)
__host__ inline bool coset_form_compiled(bool fp64, int model, int n_sym, int cs)
{
    if (model != MODEL_HC) return !fp64 && cs == n_sym && (n_sym == 2 || n_sym == 4 || n_sym == 8);
    if (fp64) return (n_sym == 4 && cs == 4) || (n_sym == 8 && cs == 4);
    return (n_sym == 2 && cs == 2) || (n_sym == 4 && (cs == 4 || cs == 2)) || (n_sym == 8 && (cs == 8 || cs == 4));
}

// operation counts with compiled FP32 kernels of the generic models (tabulated,
// IAM; the dispatch lists of dsf_k3_f32_other.cu and dsf_k3b_f32.cu): the
// tabulated ones read the form factors straight into registers (the
// runtime-count kernel stages them in shared memory), and both have the
// inversion-pair form
__host__ inline bool table_count_compiled(int n_sym) { return n_sym == 2 || n_sym == 4 || n_sym == 8; }

// per-translation-unit entries (model, multipole adjoint and ADP kind resolved at run time)
cudaError_t launch_k3_f32_hc(const K3Args &A, bool mp, bool aniso);
cudaError_t launch_k3_f32_hc_mp(const K3Args &A, bool aniso);
cudaError_t launch_k3_f32_other(const K3Args &A, int model, bool aniso);
cudaError_t launch_k3_f64(const K3Args &A, int model, bool mp, bool aniso);
cudaError_t launch_k3b_f32(const K3Args &A, int model, bool aniso);
cudaError_t launch_k3f_hc(const K3Args &A, bool aniso);
cudaError_t launch_k3f_other(const K3Args &A, int model, bool aniso);

}  // namespace dsf
