// Fused structure-factor + adjoint kernel (sm_103a), templated on precision,
// multipole derivatives, ADP kind and symmetry-operation count.
//
// One block owns one tile of up to 128 atoms (one atom per thread, atoms
// sorted by ADP kind and type so a tile holds one ADP kind and few types) and
// a contiguous chunk of reflections.  The structure keeps two resident tables
// in HBM, built once per reflection set / type update (dsf_prep_kernels.cu):
//   RS[h][s]   per (reflection, operation): h' = R^T h as integers and reals,
//              the 2^32 fixed-point phase offset h.t (or h.t for FP64), and
//              the 25 harmonics d_lm(h'/|h'|);
//   TR[t][h]   per (type, reflection): the spherical form factor and the
//              signed radial terms 4 pi N_l g_l (plus their kappa/kappa'
//              derivatives in a second table for the multipole adjoint).
// Sub-tiles of HT reflections of these tables are streamed into shared memory
// by TMA bulk copies (cp.async.bulk + mbarrier, double-buffered, bounded
// waits).  Each thread then runs the sum over operations for its atom, the
// per-reflection partial F is reduced across the block with warp shuffles and
// committed with FP64 atomics, and the per-atom derivative sums are folded
// into Kahan-compensated totals in shared memory.
//
// Reference loop restated: HansenCoppens_SF_Engine3::calculateSF_Serial*
// (src/Scattering/HansenCoppens_SF_Engine3.cpp:1030-1509, 1511-1992,
// 2649-2894) and AnyScattererStructureFactorCalculator::calculateStructure
// FactorsAndDerivatives (src/Scattering/AnyScattererStructureFactor
// Calculator.cpp:614-829).
//
// R = double: the plain form, FP64 throughout.
// R = float : the FP32-bulk form.  Phases are reduced exactly in integer
// arithmetic (fractional coordinates as 2^32 fixed point, integer h', h.t
// from integer translations in 1/24) and turned into sin/cos by a
// polynomial on the exact remainder, so no FP64 is needed per term (FP64
// runs at 1/64 of the FP32 rate on GB300).  F and the cross-block derivative
// sums are FP64.
#pragma once
#include "dsf_device.cuh"
#include "dsf_math.cuh"

namespace dsf {

template <typename R>
struct Vec2;
template <>
struct Vec2<float> { using T = float2; };
template <>
struct Vec2<double> { using T = double2; };

// one (reflection, operation) record of the RS table
template <typename R>
struct __align__(16) RsRec {
    int4 hi;   // h'0, h'1, h'2, fixed-point phase offset of h.t
    R hf[4];   // h' as reals, h.t (FP64 form)
    R y[28];   // HC: 25 harmonics, padded; other models: h'0^2, h'1^2, h'2^2, 2h'0h'1, 2h'0h'2, 2h'1h'2
};

// sin and cos of 2 pi (P 2^-32 + lo) for a phase P in 2^32 fixed point (the
// exact integer reduction mod one turn) and a small FP32 remainder lo (in
// turns).  Quadrant from the two top bits, remainder angle in [-pi/4, pi/4]
// exact in FP32 up to rounding, Taylor polynomials to degree 9 (sin) and 8
// (cos): truncation below 3e-8, so the result is limited by FP32 rounding
// (~1e-7 absolute) instead of the ~1e-6 of the hardware approximation.
__device__ __forceinline__ void sincos_fixed(uint32_t P, float lo, float *sn, float *cs)
{
    const uint32_t q = (P + 0x20000000u) >> 30;
    const int32_t r = (int32_t)(P - (q << 30));
    const float th = fmaf((float)r, 1.4629180792671596e-09f, 6.283185307179586f * lo);
    const float t2 = th * th;
    float sp = fmaf(t2, 2.7557319e-06f, -1.9841270e-04f);
    sp = fmaf(t2, sp, 8.3333333e-03f);
    sp = fmaf(t2, sp, -1.6666667e-01f);
    const float sv = fmaf(th * t2, sp, th);
    float cp = fmaf(t2, 2.4801587e-05f, -1.3888889e-03f);
    cp = fmaf(t2, cp, 4.1666668e-02f);
    cp = fmaf(t2, cp, -0.5f);
    const float cv = fmaf(t2, cp, 1.0f);
    float ss = (q & 1u) ? cv : sv;
    float cc = (q & 1u) ? sv : cv;
    if (q & 2u) ss = -ss;
    if ((q + 1u) & 2u) cc = -cc;
    *sn = ss;
    *cs = cc;
}

// temperature factor from the exponent of the ADP quadratic form: FP64 exp;
// FP32 2^x (the FP32 ADPs are stored multiplied by log2 e) by the hardware
// approximation ex2.approx.ftz.f32 alone (a few FP32 ulps: the FP32-bulk
// errors against FP64 did not change with it; x <= 0 here, and a result below
// 2^-126 flushes to zero, which moves its term by less than that)
template <typename R>
__device__ __forceinline__ R texp(R x);
template <>
__device__ __forceinline__ float texp<float>(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template <>
__device__ __forceinline__ double texp<double>(double x) { return exp(x); }

template <typename R>
__device__ __forceinline__ R shfl_xor(R v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

// ---------------------------------------------------------------------------
// TMA bulk copy + mbarrier helpers (PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of the barrier; false after ~2 s of %globaltimer,
// or after 2^26 polls whatever the timer says (the kernel then reports
// DSF_ERR_TIMEOUT instead of hanging)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < (1u << 26); it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = global_ns();
        else if ((it & 63u) == 0 && global_ns() - t0 > 2000000000ull) return false;
    }
    return false;
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------
struct SfLaunch {
    int hkl_chunk;         // reflections per block (multiple of ht)
    int ht;                // reflections per shared-memory sub-tile (multiple of 4, divides kMaxHT)
    int tile_offset;       // first tile of this launch
    int max_types;         // largest number of types in a tile of this launch
    int n_hkl_pad;         // padded reflection count of the tables (multiple of kMaxHT)
    const void *rs;        // RsRec<R> [n_hkl_pad][n_sym]
    const void *tr;        // R [n_types][n_hkl_pad][8]
    const void *trm;       // R [n_types][n_hkl_pad][8] (multipole adjoint)
    const int *cont;       // [n_hkl_pad] 1: reflection = previous one + (0,0,1) (reflections in line order)
    const int *tile_lmax;  // [n_tiles] highest l of the angular sums of the tile's atoms
    int *error;            // set to 1 on a timed-out wait
    int stall_first;       // test hook (dsf_debug_stall_next_call): the first sub-tile's copies are not issued, so
                           // its waits run out and the call returns DSF_ERR_TIMEOUT
    int coset;             // size of the sign-diagonal cosets the operations are ordered in (0: none)
};

// Operations in cosets of CS: within a coset the operations differ by a
// sign-diagonal Cartesian map diag(+-1, +-1, +-1) of the reciprocal vector.
// f[s][c] (d[s][c]) is the sign operation s gives the harmonics of parity
// class c = px + 2 py + 4 pz (parities of the harmonic in x, y, z), relative to
// the first operation of its coset.  A kernel parameter of its own: the hot
// loop reads it as immediate constant-bank operands.
struct SignTable {
    float f[8][8];
    double d[8][8];
    // the same classes for the fractional components of h' (the ADP quadratic
    // form and the position adjoint work in fractional coordinates)
    float xf[8][8];
    double xd[8][8];
};

// structures of one batched launch (sf_grad_batch3): kernel-parameter space
// holds up to kBatchItems (structure, ADP kind) items
constexpr int kBatchItems = 48;
struct SfBatchItem {
    DevStructure S;
    CallBuffers C;
    SfLaunch L;
    int n_tiles;  // tiles of this item (blocks = n_tiles x chunks)
};
struct SfBatch {
    int n;
    int block_begin[kBatchItems + 1];  // first block of each item; [n] = total
    SfBatchItem item[kBatchItems];
};

// parity class (px + 2 py + 4 pz) of the 25 harmonics of harmonic_polys
// (0: 1; 1-3: y z x; 4-8: xy yz (2zz-xx-yy) xz (xx-yy); 9-15: l = 3; 16-24: l = 4)
__host__ __device__ constexpr int harmonic_class(int q)
{
    constexpr int cls[25] = {0, 2, 4, 1, 3, 6, 0, 5, 0, 2, 7, 2, 4, 1, 4, 1, 3, 6, 3, 6, 0, 5, 0, 5, 0};
    return cls[q];
}

// the 16 (l, parity class) slots of the multipole adjoint's class sums, the
// slot of harmonic q; (l, class) of slots 0-15: (0,0) (1,2) (1,4) (1,1) (2,3)
// (2,6) (2,0) (2,5) (3,2) (3,7) (3,4) (3,1) (4,3) (4,6) (4,0) (4,5)
__host__ __device__ constexpr int harmonic_slot(int q)
{
    constexpr int sl[25] = {0, 1, 2, 3, 4, 5, 6, 7, 6, 8, 9, 8, 10, 11, 10, 11, 12, 13, 12, 13, 14, 15, 14, 15, 14};
    return sl[q];
}

// Cosets of four forming a known sign group (PAT != 0).  Within a coset ordered
// [e, a, b, ab] (signs relative to its first operation; a, b the group's
// generators as 3-bit masks of the axes they flip, PAT = a | b << 3), the sign
// operation s gives parity class c is the character chi_k(s) = (-1)^(k0 s0 +
// k1 s1) of index k = k0 + 2 k1, k0 = parity(c & a), k1 = parity(c & b), s0,
// s1 the bits of the position s.  Every signed sum over a coset's operations
// is then one of the four Walsh-Hadamard outputs of the operations' values
// (8 additions for all four), and every operation's signed combination of
// class sums one of the four outputs of the same transform of the class sums
// gathered by character.  Patterns: kPatD2 (222: a = 2z, b = 2y) and kPatC2hB
// (2/m, b unique: a = 2y, b = inversion).
constexpr int kPatD2 = 3 | (5 << 3);
constexpr int kPatC2hB = 5 | (7 << 3);

__host__ __device__ constexpr int parity3(int v) { return (v ^ (v >> 1) ^ (v >> 2)) & 1; }
__host__ __device__ constexpr int wht_char(int pat, int c)
{
    return parity3(c & pat & 7) + 2 * parity3(c & (pat >> 3) & 7);
}

// the additive identity for sums that start empty: x + (-0) = x for every x, so the compiler drops the first
// addition (x + (+0) differs from x for x = -0, and is kept)
template <typename R>
constexpr R kZero = R(-0.0);

// W[k] = sum_s chi_k(s) u[s] for the coset order [e, a, b, ab] (the transform is its own inverse up to 1/4,
// and symmetric: the same butterfly gives each operation's combination of the character sums)
template <typename R>
__device__ __forceinline__ void wht4(const R (&u)[4], R (&W)[4])
{
    const R t0 = u[0] + u[1], t1 = u[0] - u[1], t2 = u[2] + u[3], t3 = u[2] - u[3];
    W[0] = t0 + t2;
    W[1] = t1 + t3;
    W[2] = t0 - t2;
    W[3] = t1 - t3;
}

// two transforms at once (the real and imaginary parts of a complex quantity, or two real ones): in FP32 as
// packed pairs (one add.f32x2 or fma.f32x2 per butterfly leg instead of two scalar adds; a - b as fma(b, -1, a),
// rounded once like the subtraction, so the results equal the scalar form's)
template <typename R>
__device__ __forceinline__ void wht4x2(const R (&a)[4], const R (&b)[4], R (&A)[4], R (&B)[4])
{
    if constexpr (sizeof(R) == 4) {
        const float2 m1 = make_float2(-1.f, -1.f);
        const float2 u0 = make_float2(a[0], b[0]), u1 = make_float2(a[1], b[1]);
        const float2 u2 = make_float2(a[2], b[2]), u3 = make_float2(a[3], b[3]);
        const float2 t0 = __fadd2_rn(u0, u1), t1 = __ffma2_rn(u1, m1, u0);
        const float2 t2 = __fadd2_rn(u2, u3), t3 = __ffma2_rn(u3, m1, u2);
        const float2 w0 = __fadd2_rn(t0, t2), w1 = __fadd2_rn(t1, t3);
        const float2 w2 = __ffma2_rn(t2, m1, t0), w3 = __ffma2_rn(t3, m1, t1);
        A[0] = w0.x; A[1] = w1.x; A[2] = w2.x; A[3] = w3.x;
        B[0] = w0.y; B[1] = w1.y; B[2] = w2.y; B[3] = w3.y;
    } else {
        wht4(a, A);
        wht4(b, B);
    }
}

// one table row of a column: its NR operation values (complex64, contiguous, 16 x NR-byte aligned), streamed
// past L1 (read once): 256-bit loads for four operations
template <int NR>
__device__ __forceinline__ void ld_table_row(const float2 *p, float2 *d)
{
    if constexpr (NR % 4 == 0) {
#pragma unroll
        for (int k = 0; k < NR / 4; k++) {
            float v[8];
            asm("ld.global.cs.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                : "l"(p + 4 * k));
#pragma unroll
            for (int q = 0; q < 4; q++) d[4 * k + q] = make_float2(v[2 * q], v[2 * q + 1]);
        }
    } else if constexpr (NR == 2) {
        const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
        d[0] = make_float2(v.x, v.y);
        d[1] = make_float2(v.z, v.w);
    } else {
#pragma unroll
        for (int q = 0; q < NR; q++) d[q] = __ldcs(p + q);
    }
}

template <typename R>
struct StageLayout {
    size_t rs, tr, trm, gw, h2, cont, tab, bytes;
    // tab: FP32 tabulated model, the tile's form factors [ht][kTileAtoms][ns] (complex64)
    __host__ __device__ StageLayout(int ht, int ns, int max_types, bool mp, bool table = false)
    {
        tab = 0;
        rs = (table && sizeof(R) == 4) ? sizeof(float2) * (size_t)ht * ns * kTileAtoms : 0;
        tr = rs + sizeof(RsRec<R>) * (size_t)ht * ns;
        trm = tr + sizeof(R) * 8 * (size_t)ht * max_types;
        gw = trm + (mp ? sizeof(R) * 8 * (size_t)ht * max_types : 0);
        h2 = gw + sizeof(R) * 2 * (size_t)ht;
        cont = h2 + sizeof(R) * (size_t)ht;
        bytes = cont + sizeof(int) * (size_t)ht;
        bytes = (bytes + 15) & ~(size_t)15;
    }
};

template <typename R, bool MP>
__host__ __device__ constexpr int n_channels() { return MP ? 38 : 10; }

template <typename R, bool MP>
__host__ __device__ inline size_t sf_smem_bytes(int ht, int ns, int max_types, bool table = false)
{
    StageLayout<R> L(ht, ns, max_types, MP, table);
    size_t b = 64;                                                        // barriers
    b += 2 * L.bytes;                                                     // two stages
    b += sizeof(R) * 2 * (size_t)(kTileAtoms / 32) * ht;                  // warp partials of F
    b += sizeof(R) * 2 * (size_t)n_channels<R, MP>() * kTileAtoms;        // Kahan totals
    b += sizeof(int) * kMaxTileTypes;
    return b;
}

// e^{2 pi i phi}: FP32 from the fixed-point phase, FP64 from h'.x + h.t reduced mod 1
template <typename R>
struct PhaseOps;
template <>
struct PhaseOps<float> {
    static __device__ __forceinline__ void exact(const RsRec<float> &rec, uint32_t xq0, uint32_t xq1, uint32_t xq2,
                                                 float x0, float x1, float x2, float *sn, float *cs)
    {
        const int4 hi = rec.hi;
        const uint32_t P = (uint32_t)hi.x * xq0 + (uint32_t)hi.y * xq1 + (uint32_t)hi.z * xq2 + (uint32_t)hi.w;
        sincos_fixed(P, rec.hf[0] * x0 + rec.hf[1] * x1 + rec.hf[2] * x2, sn, cs);
    }
};
template <>
struct PhaseOps<double> {
    static __device__ __forceinline__ void exact(const RsRec<double> &rec, uint32_t, uint32_t, uint32_t, double x0,
                                                 double x1, double x2, double *sn, double *cs)
    {
        double ph = rec.hf[0] * x0 + rec.hf[1] * x1 + rec.hf[2] * x2 + rec.hf[3];
        ph -= rint(ph);
        sincospi(2.0 * ph, sn, cs);
    }
};

// Reflections that continue a lattice line (h, k, l) -> (h, k, l+1) get their
// phase factors by one complex multiplication with the per-atom, per-operation
// step e^{2 pi i ((R^T e_l).x + e_l.t)} (the reference engine's line
// recurrence, scattering_utilities::calculate_line_phase_factors,
// src/Scattering/scattering_utilities.cpp:575-627); the exact phase is
// re-anchored at every line start, at every sub-tile start and, in the FP32
// form, every kAnchorF32 reflections so the FP32 rounding of the step cannot
// build up.  With 16 (sub-tiles hold at most 16 reflections: an anchor at
// every line and sub-tile start) the FP32 error against FP64 measured
// 3.6e-7 (F) on the 5,000-atom P2_1 2_1 2_1 and 50,000-atom P4_3 2_1 2
// structures and 2.2e-7 on a 256-crystal P2_1/c tabulated batch, against
// 3.1-3.2e-7 and 1.6e-7 with 8, for 2.4-3.4% of the time.
constexpr int kAnchorF32 = 16;

// GRAD = false: structure factors only (the reference's calculateStructureFactors, which runs its engine with
// every derivative switched off, HansenCoppensStructureFactorCalculator.cpp:305-326): the derivative sums are
// never stored, so the compiler drops the whole adjoint
// INV = true (FP32 tabulated and IAM models, the caller's operations as n/2 operations followed by their
// images under an inversion at the origin, x -> -R x - t): the images' phase factors are the conjugates of their
// partners' and their temperature factors equal, so only half the operations run the phase and exp work
// PAT != 0 (CS = 4): the coset's operations in the order [e, a, b, ab] of that sign group, the signed sums by
// Walsh-Hadamard transforms (wht4) instead of per-operation sign multiply-adds
template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS, bool GRAD = true, bool INV = false,
          int PAT = 0>
__device__ __forceinline__ void sf_grad_body(const DevStructure &S, const CallBuffers &C, const SfLaunch &L,
                                             const SignTable &G, const int tile_rel, const int chunk)
{
    // CS > 0 (HC, fixed operation count, operations in sign-diagonal cosets of
    // CS): the angular sums are formed once per (atom, reflection, coset) by
    // parity class from the harmonics of the coset's first operation, and each
    // operation combines the eight class sums with its signs -- the same sums
    // as the per-operation form
    // The ADP side of the coset form (all models, ANISO): within a coset h' of
    // operation s is a sign-diagonal image of the first operation's h', so the
    // quadratic form is q_s = q_diag + signed cross terms, and the position and
    // ADP adjoints need six signed sums of u per coset instead of h' and m6 per
    // operation (ADIAG).
    // The position adjoint in the coset form (XDIAG): the fractional h' of operation s is
    // the coset's first h' with signs, so the x, y, z adjoint sums are the first h' times
    // three signed sums of u per coset.
    constexpr bool DIAG = CS > 0 && MODEL == MODEL_HC;
    constexpr bool ADIAG = CS > 0 && ANISO;
    constexpr bool XDIAG = CS > 0;
    constexpr int NSG = ADIAG ? 6 : (XDIAG ? 3 : 1);  // signed sums of u per coset
    constexpr bool WHT = PAT != 0 && CS == 4;
    static_assert(PAT == 0 || CS == 4, "sign-group patterns: cosets of four");
    static_assert(CS == 0 || (NSC > 0 && NSC <= 8 && NSC % CS == 0), "coset form: compiled count <= 8");
    static_assert(GRAD || !MP, "the multipole adjoint needs the derivative pass");
    static_assert(!INV || (MODEL != MODEL_HC && NSC > 0 && NSC % 2 == 0), "inversion pairs: generic models, even count");
    using R2 = typename Vec2<R>::T;
    constexpr bool F32 = sizeof(R) == 4;
    constexpr int NT = n_channels<R, MP>();
    constexpr int kWarps = kTileAtoms / 32;
    constexpr bool HC = MODEL == MODEL_HC;
    constexpr bool TABLE = MODEL == MODEL_TABLE;
    constexpr bool REC = NSC > 0;                 // line recurrence (register arrays need a fixed count)
    constexpr int NR = NSC > 0 ? NSC : 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nS = NSC > 0 ? NSC : S.n_sym;
    const int ht = L.ht;
    const int tile = L.tile_offset + tile_rel;
    const int h_begin = chunk * L.hkl_chunk;
    const int h_end = min(S.n_hkl, h_begin + L.hkl_chunk);
    if (h_begin >= h_end) return;
    const int a_begin = S.tile_begin[tile], a_end = S.tile_begin[tile + 1];
    const int nT = S.tile_ntypes[tile];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool high_l = HC && L.tile_lmax[tile] >= 3;  // uniform over the block

    // shared memory carve-up
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);  // [2]
    // FP32 tabulated form factors: with a compiled operation count each thread
    // loads its own column of the next group of four reflections into registers
    // while the current group runs (coalesced streaming loads, no shared memory,
    // so the sub-tiles stay long); otherwise they are staged by bulk copies
    constexpr bool TAB_REG = TABLE && F32 && NSC > 0;
    // the four reflections of a group as a loop (one copy of the reflection
    // body: kernels with eight unrolled operations or the multipole adjoint
    // otherwise outgrow the instruction cache) or unrolled (small bodies, and
    // the register-held form factors, which need a compile-time index)
    constexpr bool ROLL_J = !TAB_REG && (NSC > 4 || MP);
    constexpr bool TAB_SMEM = TABLE && F32 && NSC == 0;
    const StageLayout<R> SL(ht, nS, L.max_types, MP, TAB_SMEM);
    unsigned char *stage0 = smem_raw + 64;
    R2 *sF = reinterpret_cast<R2 *>(stage0 + 2 * SL.bytes);           // [kWarps][ht]
    R *sTot = reinterpret_cast<R *>(sF + kWarps * ht);                 // [NT][kTileAtoms]
    R *sCmp = sTot + NT * kTileAtoms;                                   // [NT][kTileAtoms]
    int *sTypes = reinterpret_cast<int *>(sCmp + NT * kTileAtoms);     // [nT]

    for (int i = tid; i < nT; i += blockDim.x) sTypes[i] = S.tile_types[tile * kMaxTileTypes + i];
    if constexpr (GRAD)
        for (int q = 0; q < NT; q++) {
            sTot[q * kTileAtoms + tid] = R(0);
            sCmp[q * kTileAtoms + tid] = R(0);
        }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();

    const RsRec<R> *rs_g = reinterpret_cast<const RsRec<R> *>(L.rs);
    const R *tr_g = reinterpret_cast<const R *>(L.tr);
    const R *trm_g = reinterpret_cast<const R *>(L.trm);
    const R2 *gw_g;
    const R *h2_g;
    if constexpr (F32) {
        gw_g = C.gw_f;
        h2_g = S.h2f;
    } else {
        gw_g = C.gw_d;
        h2_g = S.h2;
    }

    // thread 0 streams a sub-tile of the tables into one stage buffer
    auto issue = [&](int buf, int h0) {
        unsigned char *st = stage0 + buf * SL.bytes;
        const uint32_t rs_bytes = (uint32_t)(sizeof(RsRec<R>) * ht * nS);
        const uint32_t tr_bytes = (uint32_t)(sizeof(R) * 8 * ht);
        // the tile's columns of one table row (each column its nS operation values): 16-byte aligned (even
        // first column, even row stride), rounded up to 16 bytes (the table has 16 bytes of slack at its end)
        const int tab_col0 = a_begin + (a_begin >= S.table_split ? S.table_shift : 0);
        const uint32_t tab_bytes = (uint32_t)((sizeof(float2) * (size_t)nS * (a_end - a_begin) + 15) & ~(size_t)15);
        const uint32_t bytes = rs_bytes + (uint32_t)(2 * sizeof(R) * ht) + (uint32_t)(sizeof(R) * ht) +
                               (uint32_t)(sizeof(int) * ht) + (TABLE ? 0u : tr_bytes * nT * (MP ? 2u : 1u)) +
                               (TAB_SMEM ? tab_bytes * (uint32_t)ht : 0u);
        fence_proxy_async();
        mbar_expect_tx(&bar[buf], bytes);
        if constexpr (TAB_SMEM) {
            for (int q = 0; q < ht; q++)
                bulk_copy(st + SL.tab + sizeof(float2) * kTileAtoms * (size_t)(q * nS),
                          S.table_f + ((size_t)(h0 + q) * S.table_stride + tab_col0) * nS, tab_bytes, &bar[buf]);
        }
        bulk_copy(st + SL.rs, rs_g + (size_t)h0 * nS, rs_bytes, &bar[buf]);
        if constexpr (!TABLE) {
            for (int t = 0; t < nT; t++) {
                const size_t row = ((size_t)sTypes[t] * L.n_hkl_pad + h0) * 8;
                bulk_copy(st + SL.tr + (size_t)tr_bytes * t, tr_g + row, tr_bytes, &bar[buf]);
                if constexpr (MP) bulk_copy(st + SL.trm + (size_t)tr_bytes * t, trm_g + row, tr_bytes, &bar[buf]);
            }
        }
        bulk_copy(st + SL.gw, gw_g + h0, (uint32_t)(2 * sizeof(R) * ht), &bar[buf]);
        bulk_copy(st + SL.h2, h2_g + h0, (uint32_t)(sizeof(R) * ht), &bar[buf]);
        bulk_copy(st + SL.cont, L.cont + h0, (uint32_t)(sizeof(int) * ht), &bar[buf]);
    };

    // per-atom registers
    const int a = a_begin + tid;
    const bool have = a < a_end;
    bool active = false;
    int lt = 0;
    R w = R(0), pg[HC ? 25 : 1], adp[ANISO ? 6 : 1];
    R anre = R(0), anim = R(0);
    uint32_t xq0 = 0, xq1 = 0, xq2 = 0;
    R x0 = R(0), x1 = R(0), x2 = R(0);  // FP32: low parts (turns); FP64: coordinates
    bool has_adp = false;
    R step_re[NR], step_im[NR], e_re[NR], e_im[NR];
#pragma unroll
    for (int q = 0; q < NR; q++) { step_re[q] = R(1); step_im[q] = R(0); e_re[q] = R(1); e_im[q] = R(0); }
#pragma unroll
    for (int q = 0; q < (HC ? 25 : 1); q++) pg[q] = R(0);
#pragma unroll
    for (int q = 0; q < (ANISO ? 6 : 1); q++) adp[q] = R(0);
    if (have) {
        active = S.atom_active[a] != 0;
        lt = S.atom_ltype[a];
        has_adp = S.atom_adpk[a] != 0;
        if constexpr (F32) {
            w = S.atom_w_f[a];
            const float2 an = S.atom_anom_f[a];
            anre = an.x; anim = an.y;
            xq0 = S.atom_xq[3 * a]; xq1 = S.atom_xq[3 * a + 1]; xq2 = S.atom_xq[3 * a + 2];
            x0 = S.atom_xlo[3 * a]; x1 = S.atom_xlo[3 * a + 1]; x2 = S.atom_xlo[3 * a + 2];
#pragma unroll
            for (int q = 0; q < (ANISO ? 6 : 1); q++) adp[q] = S.atom_adp_f[6 * a + q];
            if constexpr (HC)
#pragma unroll
                for (int q = 0; q < 25; q++) pg[q] = S.atom_pg_f[25 * a + q];
        } else {
            w = S.atom_w_d[a];
            const double2 an = S.atom_anom_d[a];
            anre = an.x; anim = an.y;
            x0 = S.atom_xd[3 * a]; x1 = S.atom_xd[3 * a + 1]; x2 = S.atom_xd[3 * a + 2];
#pragma unroll
            for (int q = 0; q < (ANISO ? 6 : 1); q++) adp[q] = S.atom_adp_d[6 * a + q];
            if constexpr (HC)
#pragma unroll
                for (int q = 0; q < 25; q++) pg[q] = S.atom_pg_d[25 * a + q];
        }
        if constexpr (REC) {
            // line steps (computed in FP64 with the atom conversion, once per atom upload)
#pragma unroll
            for (int s = 0; s < (INV ? NR / 2 : NR); s++) {  // INV: the images need no line steps
                if constexpr (F32) {
                    const float2 st = S.atom_step_f[(size_t)a * NR + s];
                    step_re[s] = st.x;
                    step_im[s] = st.y;
                } else {
                    const double2 st = S.atom_step_d[(size_t)a * NR + s];
                    step_re[s] = st.x;
                    step_im[s] = st.y;
                }
            }
        }
    }

    // TAB_REG: form factors of the current and the next group of four reflections
    constexpr int kTabN = TAB_REG ? 4 * NR : 1;
    float2 tab_a[kTabN], tab_b[kTabN];
    const float2 *tab_col = nullptr;
    if constexpr (TAB_REG) {
        // a tile's columns are contiguous (tiles do not straddle table_split); row 0 of this atom's column
        tab_col = S.table_f + (size_t)(a + (a >= S.table_split ? S.table_shift : 0)) * NR;
#pragma unroll
        for (int q = 0; q < 4 * NR; q++) tab_a[q] = tab_b[q] = make_float2(0.f, 0.f);
    }
    // rows hg .. hg + 3 (below n_hkl_pad for every group that starts before h_end): per row the column's NR
    // operation values, contiguous (one 32-byte load per four operations)
    auto tab_load = [&](float2 (&dst)[kTabN], int hg) {
        if constexpr (TAB_REG) {
            if (have && hg < h_end) {
                const size_t rstep = (size_t)S.table_stride * NR;
#pragma unroll
                for (int j = 0; j < 4; j++) ld_table_row<NR>(tab_col + (size_t)(hg + j) * rstep, &dst[j * NR]);
            }
        }
    };
    tab_load(tab_b, h_begin);

    if (tid == 0 && !L.stall_first) issue(0, h_begin);
    uint32_t parity[2] = {0u, 0u};
    int k = 0;
    // per-thread partial derivative sums, folded into the compensated totals
    // every `fold` sub-tiles (about 32 reflections)
    R part[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) part[q] = R(0);
    const int fold = ht >= 32 ? 1 : 32 / ht;
    for (int h0 = h_begin; h0 < h_end; h0 += ht, k++) {
        const int buf = k & 1;
        if (tid == 0 && h0 + ht < h_end) issue(buf ^ 1, h0 + ht);
        const uint32_t phase = parity[buf];
        const bool ok = mbar_wait(&bar[buf], phase);
        parity[buf] ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(L.error, 1);
                // bounded: let this sub-tile's copies and the next one's (if issued) land first
                mbar_wait(&bar[buf], phase);
                if (h0 + ht < h_end) mbar_wait(&bar[buf ^ 1], parity[buf ^ 1]);
            }
            return;
        }
        const unsigned char *st = stage0 + buf * SL.bytes;
        const RsRec<R> *sRs = reinterpret_cast<const RsRec<R> *>(st + SL.rs);
        const R *sTr = reinterpret_cast<const R *>(st + SL.tr);
        const R *sTrm = reinterpret_cast<const R *>(st + SL.trm);
        const R2 *sG = reinterpret_cast<const R2 *>(st + SL.gw);
        const R *sH2 = reinterpret_cast<const R *>(st + SL.h2);
        const int *sCont = reinterpret_cast<const int *>(st + SL.cont);

        // reflections in groups of four: the partial F of a group is reduced across
        // the warp by one butterfly reduce-scatter of its eight values.  TAB_REG: the
        // group's form factors in `cur` while the next group's load into `nxt`
        auto group = [&](const int g0, float2 (&cur)[kTabN], float2 (&nxt)[kTabN]) {
            if constexpr (TAB_REG) tab_load(nxt, h0 + g0 + 4);
            R Fv[8];
#pragma unroll
            for (int q = 0; q < 8; q++) Fv[q] = R(0);
            // reflection j of the group; its partial F goes to Fv[2j], Fv[2j + 1]
            auto reflection = [&](const int j) {
                const int hl = g0 + j;
                const bool anchor = !REC || sCont[hl] == 0 || hl == 0 ||
                                    (F32 && (hl % kAnchorF32) == 0);
                if (active) {
                    const R2 g = sG[hl];
                    R fsre = anre, fsim = anim, r0 = 0, r1 = 0, r2 = 0, r3 = 0, r4 = 0;
                    const R *rad = sTr + (size_t)(lt * ht + hl) * 8;
                    if constexpr (!TABLE) {
                        // rows of 8 values, 32-byte aligned (16-byte stage offsets, 16-byte record sizes)
                        if constexpr (F32) {
                            const float4 ra = reinterpret_cast<const float4 *>(rad)[0];
                            const float2 rb = reinterpret_cast<const float2 *>(rad)[2];
                            fsre += ra.x;
                            r0 = ra.y; r1 = ra.z; r2 = ra.w; r3 = rb.x; r4 = rb.y;
                        } else {
                            const double2 ra = reinterpret_cast<const double2 *>(rad)[0];
                            const double2 rb = reinterpret_cast<const double2 *>(rad)[1];
                            const double2 rc = reinterpret_cast<const double2 *>(rad)[2];
                            fsre += ra.x;
                            r0 = ra.y; r1 = rb.x; r2 = rb.y; r3 = rc.x; r4 = rc.y;
                        }
                    }
                    R Tiso = R(1);
                    if (!ANISO && has_adp) Tiso = texp<R>(-adp[0] * sH2[hl]);
                    const R gre = g.x * Tiso, gim = g.y * Tiso;  // adjoint weight with the isotropic factor
                    R Ure = kZero<R>, Uim = kZero<R>;
                    R Xre[3] = {0, 0, 0}, Xim[3] = {0, 0, 0};
                    R Are[ANISO ? 6 : 1], Aim[ANISO ? 6 : 1];
#pragma unroll
                    for (int q = 0; q < (ANISO ? 6 : 1); q++) { Are[q] = R(0); Aim[q] = R(0); }
                    R Ere = 0, Eim = 0, Kre = 0, Kim = 0;
                    const RsRec<R> *recs = sRs + (size_t)hl * nS;
                    // XDIAG: the coset's first h' and the signed sums of u: x y z (classes 1 2 4);
                    // ADIAG adds its m6, the split quadratic form, the signed sums xy xz yz
                    // (classes 3 5 6) and plain U
                    R hr[3] = {0, 0, 0}, m6r[ADIAG ? 6 : 1], qd = 0, qc[3] = {0, 0, 0}, qw[WHT && ADIAG ? 4 : 1];
                    R Sre[NSG], Sim[NSG], Ucre = 0, Ucim = 0;
                    R gUc = kZero<R>;  // WHT: Re(g U), contracted per coset
#pragma unroll
                    for (int q = 0; q < (ADIAG ? 6 : 1); q++) m6r[q] = R(0);
#pragma unroll
                    for (int q = 0; q < NSG; q++) { Sre[q] = R(0); Sim[q] = R(0); }
                    auto adp_coset_begin = [&](const RsRec<R> &rec) {
                        if constexpr (XDIAG) {
                            hr[0] = rec.hf[0]; hr[1] = rec.hf[1]; hr[2] = rec.hf[2];
#pragma unroll
                            for (int q = 0; q < NSG; q++) { Sre[q] = R(0); Sim[q] = R(0); }
                        }
                        if constexpr (ADIAG) {
                            if constexpr (HC) {
                                m6r[0] = hr[0] * hr[0]; m6r[1] = hr[1] * hr[1]; m6r[2] = hr[2] * hr[2];
                                m6r[3] = R(2) * hr[0] * hr[1]; m6r[4] = R(2) * hr[0] * hr[2];
                                m6r[5] = R(2) * hr[1] * hr[2];
                            } else {
                                // the same six products, from the record (rs_prep_kernel; the other models
                                // have no harmonics there)
#pragma unroll
                                for (int q = 0; q < 6; q++) m6r[q] = rec.y[q];
                            }
                            qd = adp[0] * m6r[0] + adp[1] * m6r[1] + adp[2] * m6r[2];
                            qc[0] = adp[3] * m6r[3]; qc[1] = adp[4] * m6r[4]; qc[2] = adp[5] * m6r[5];
                            Ucre = R(0); Ucim = R(0);
                            if constexpr (WHT) {
                                // each operation's quadratic form: qd + the cross terms xy xz yz with its signs
                                R Qp[4] = {qd, kZero<R>, kZero<R>, kZero<R>};
                                Qp[wht_char(PAT, 3)] += qc[0];
                                Qp[wht_char(PAT, 5)] += qc[1];
                                Qp[wht_char(PAT, 6)] += qc[2];
                                wht4(Qp, qw);
                            }
                        }
                    };
                    auto adp_coset_end = [&]() {
                        if constexpr (WHT) {
                            // contracted in wht_end
                        } else if constexpr (XDIAG) {
#pragma unroll
                            for (int c = 0; c < 3; c++) { Xre[c] += hr[c] * Sre[c]; Xim[c] += hr[c] * Sim[c]; }
                        }
                        if constexpr (ADIAG && !WHT) {
#pragma unroll
                            for (int q = 0; q < 3; q++) { Are[q] -= m6r[q] * Ucre; Aim[q] -= m6r[q] * Ucim; }
#pragma unroll
                            for (int q = 3; q < 6; q++) { Are[q] -= m6r[q] * Sre[q]; Aim[q] -= m6r[q] * Sim[q]; }
                        }
                    };
                    // coset form: radial-weighted class sums, even l (real part) and odd l (imaginary part)
                    R Ec[4] = {0, 0, 0, 0}, Oc[4] = {0, 0, 0, 0};  // classes 0 3 6 5 | 2 4 1 7
                    // WHT: per position of the coset, the operations' f (HC), u and (multipole adjoint) g z
                    R fwr[WHT ? 4 : 1], fwi[WHT ? 4 : 1], ur4[WHT ? 4 : 1], ui4[WHT ? 4 : 1];
                    R wr4[WHT && MP ? 4 : 1], wi4[WHT && MP ? 4 : 1];
                    // WHT (HC): each operation's f from the class sums gathered by character
                    auto forward_wht = [&]() {
                        if constexpr (WHT && DIAG) {
                            constexpr int ec[4] = {0, 3, 6, 5}, oc[4] = {2, 4, 1, 7};
                            R Ep[4] = {kZero<R>, kZero<R>, kZero<R>, kZero<R>}, t[4];
                            R Op[4] = {kZero<R>, kZero<R>, kZero<R>, kZero<R>};
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                Ep[wht_char(PAT, ec[q])] += Ec[q];
                                Op[wht_char(PAT, oc[q])] += Oc[q];
                            }
                            wht4x2(Ep, Op, fwr, t);
#pragma unroll
                            for (int q = 0; q < 4; q++) fwi[q] = fsim + t[q];
                        }
                    };
                    // with the multipole adjoint: the same class sums weighted by the kappa'
                    // derivatives of the radial terms (De, Do), and the operations' signed
                    // adjoint weights per class (We: Re(g z) of the even classes, Wo: Im(g z) of
                    // the odd ones), folded into the P_lm channels once per coset: the weight of
                    // harmonic (l, c) is r_l We[c] (even l) or -r_l Wo[c] (odd l)
                    R De[DIAG && MP ? 4 : 1], Do[DIAG && MP ? 4 : 1], We[DIAG && MP ? 4 : 1], Wo[DIAG && MP ? 4 : 1];
#pragma unroll
                    for (int k = 0; k < (DIAG && MP ? 4 : 1); k++) { De[k] = Do[k] = We[k] = Wo[k] = R(0); }
                    // WHT: the coset's sums from its four operations' values: U (character 0), the signed sums
                    // of u by the fractional classes x y z (xy xz yz), and the multipole adjoint's class weights
                    auto wht_end = [&]() {
                        if constexpr (WHT) {
                            R Wr[4], Wi[4];
                            wht4x2(ur4, ui4, Wr, Wi);
                            Ure += Wr[0];
                            Uim += Wi[0];
                            constexpr int cls[6] = {1, 2, 4, 3, 5, 6};
                            if constexpr (GRAD) {
                                // the position and ADP adjoints contracted with g here, once per coset, from
                                // the characters their classes take: -h'_c Im(g S_c) and -m6_q Re(g S_q)
                                // (the diagonal q with S = U of the coset); Re(g U) summed over the cosets
                                const R gw0 = gre * Wr[0] - gim * Wi[0];
                                gUc += gw0;
#pragma unroll
                                for (int c = 0; c < 3; c++) {
                                    const int k = wht_char(PAT, cls[c]);
                                    part[CH_XYZ + c] -= hr[c] * (gre * Wi[k] + gim * Wr[k]);
                                }
                                if constexpr (ADIAG) {
#pragma unroll
                                    for (int q = 0; q < 3; q++) part[CH_ADP + q] -= m6r[q] * gw0;
#pragma unroll
                                    for (int q = 3; q < 6; q++) {
                                        const int k = wht_char(PAT, cls[q]);
                                        part[CH_ADP + q] -= m6r[q] * (gre * Wr[k] - gim * Wi[k]);
                                    }
                                }
                            }
                            if constexpr (MP && DIAG) {
                                R Vr[4], Vi[4];
                                wht4x2(wr4, wi4, Vr, Vi);
                                We[0] = Vr[0]; We[1] = Vr[wht_char(PAT, 3)]; We[2] = Vr[wht_char(PAT, 6)];
                                We[3] = Vr[wht_char(PAT, 5)];
                                Wo[0] = Vi[wht_char(PAT, 2)]; Wo[1] = Vi[wht_char(PAT, 4)]; Wo[2] = Vi[wht_char(PAT, 1)];
                                Wo[3] = Vi[wht_char(PAT, 7)];
                            }
                        }
                    };
                    auto mp_coset_begin = [&](const R *y, const R *dr) {
                        if constexpr (DIAG && MP) {
                            // unweighted slot sums (l, class) of the coset's first operation
                            R Acl[16];
#pragma unroll
                            for (int k = 0; k < 16; k++) Acl[k] = R(0);
#pragma unroll
                            for (int q = 0; q < 9; q++) Acl[harmonic_slot(q)] += pg[q] * y[q];
                            Ec[0] = fsre + r0 * Acl[0] + r2 * Acl[6];
                            Ec[1] = r2 * Acl[4];
                            Ec[2] = r2 * Acl[5];
                            Ec[3] = r2 * Acl[7];
                            Oc[0] = r1 * Acl[1];
                            Oc[1] = r1 * Acl[2];
                            Oc[2] = r1 * Acl[3];
                            Oc[3] = R(0);
                            De[0] = dr[2] * Acl[0] + dr[4] * Acl[6];
                            De[1] = dr[4] * Acl[4];
                            De[2] = dr[4] * Acl[5];
                            De[3] = dr[4] * Acl[7];
                            Do[0] = dr[3] * Acl[1];
                            Do[1] = dr[3] * Acl[2];
                            Do[2] = dr[3] * Acl[3];
                            Do[3] = R(0);
                            if (high_l) {
#pragma unroll
                                for (int q = 9; q < 25; q++) Acl[harmonic_slot(q)] += pg[q] * y[q];
                                Ec[0] += r4 * Acl[14]; Ec[1] += r4 * Acl[12]; Ec[2] += r4 * Acl[13]; Ec[3] += r4 * Acl[15];
                                Oc[0] += r3 * Acl[8]; Oc[1] += r3 * Acl[10]; Oc[2] += r3 * Acl[11]; Oc[3] = r3 * Acl[9];
                                De[0] += dr[6] * Acl[14]; De[1] += dr[6] * Acl[12]; De[2] += dr[6] * Acl[13];
                                De[3] += dr[6] * Acl[15];
                                Do[0] += dr[5] * Acl[8]; Do[1] += dr[5] * Acl[10]; Do[2] += dr[5] * Acl[11];
                                Do[3] = dr[5] * Acl[9];
                            }
#pragma unroll
                            for (int k = 0; k < 4; k++) { We[k] = R(0); Wo[k] = R(0); }
                        }
                    };
                    auto flush_slots = [&](const R *y, const R *dr) {
                        if constexpr (DIAG && MP) {
                            // P_val and kappa: Re(g sum_s z_s T) dr_0,1 = We[0] dr_0,1; kappa':
                            // sum_s Re(g z_s T (dre_s + i dim_s)) with dre_s = sum_c sign_c(s) De[c]
                            // (dim_s likewise) = sum_c De[c] We[c] - Do[c] Wo[c]
                            part[CH_PV] += dr[0] * We[0];
                            part[CH_KAPPA] += dr[1] * We[0];
                            part[CH_KAPPA_P] += De[0] * We[0] + De[1] * We[1] + De[2] * We[2] + De[3] * We[3] -
                                                (Do[0] * Wo[0] + Do[1] * Wo[1] + Do[2] * Wo[2] + Do[3] * Wo[3]);
                            // slot weights in harmonic_slot order
                            const R QC[16] = {r0 * We[0], -r1 * Wo[0], -r1 * Wo[1], -r1 * Wo[2],
                                              r2 * We[1], r2 * We[2], r2 * We[0], r2 * We[3],
                                              -r3 * Wo[0], -r3 * Wo[3], -r3 * Wo[1], -r3 * Wo[2],
                                              r4 * We[1], r4 * We[2], r4 * We[0], r4 * We[3]};
#pragma unroll
                            for (int q = 0; q < 25; q++) part[CH_PLM + q] += QC[harmonic_slot(q)] * y[q];
                        }
                    };
                    auto class_sums = [&](const R *y) {
                        if constexpr (DIAG && !MP) {
                        Oc[3] = R(0);
                        Ec[0] = fsre + r0 * (pg[0] * y[0]) + r2 * (pg[6] * y[6] + pg[8] * y[8]);
                        Ec[1] = r2 * (pg[4] * y[4]);
                        Ec[2] = r2 * (pg[5] * y[5]);
                        Ec[3] = r2 * (pg[7] * y[7]);
                        Oc[0] = r1 * (pg[1] * y[1]);
                        Oc[1] = r1 * (pg[2] * y[2]);
                        Oc[2] = r1 * (pg[3] * y[3]);
                        if (high_l) {
                            Ec[0] += r4 * (pg[20] * y[20] + pg[22] * y[22] + pg[24] * y[24]);
                            Ec[1] += r4 * (pg[16] * y[16] + pg[18] * y[18]);
                            Ec[2] += r4 * (pg[17] * y[17] + pg[19] * y[19]);
                            Ec[3] += r4 * (pg[21] * y[21] + pg[23] * y[23]);
                            Oc[0] += r3 * (pg[9] * y[9] + pg[11] * y[11]);
                            Oc[1] += r3 * (pg[12] * y[12] + pg[14] * y[14]);
                            Oc[2] += r3 * (pg[13] * y[13] + pg[15] * y[15]);
                            Oc[3] = r3 * (pg[10] * y[10]);
                        }
                        }
                    };
                    // INV: e^{i theta} T of the first half of the operations, for their inversion images
                    R zT_re[INV ? NR / 2 : 1] = {}, zT_im[INV ? NR / 2 : 1] = {};  // each set before its image reads it
                    auto term = [&](int s) {
                        const RsRec<R> &rec = recs[s];
                        const R h0f = rec.hf[0], h1f = rec.hf[1], h2f = rec.hf[2];
                        R zre, zim;  // e^{i theta} T_s
                        R m6[ANISO ? 6 : 1];
                        if constexpr (ANISO && !ADIAG) {
                            m6[0] = h0f * h0f; m6[1] = h1f * h1f; m6[2] = h2f * h2f;
                            m6[3] = R(2) * h0f * h1f; m6[4] = R(2) * h0f * h2f; m6[5] = R(2) * h1f * h2f;
                        }
                        const auto xs = [&](int c) -> R {
                            if constexpr (F32) return G.xf[s][c]; else return G.xd[s][c];
                        };
                        bool image = false;
                        if constexpr (INV) image = s >= NR / 2;
                        if (image) {
                            // the inversion image of operation s - n/2 (inversion at the origin): h' -> -h',
                            // the same translation sign-reversed, so the conjugate phase and the same T
                            if constexpr (INV) {
                                zre = zT_re[s - NR / 2];
                                zim = -zT_im[s - NR / 2];
                            }
                        } else {
                            R cs, sn;
                            if constexpr (REC) {
                                if (anchor) {
                                    PhaseOps<R>::exact(rec, xq0, xq1, xq2, x0, x1, x2, &sn, &cs);
                                } else {
                                    cs = e_re[s] * step_re[s] - e_im[s] * step_im[s];
                                    sn = e_re[s] * step_im[s] + e_im[s] * step_re[s];
                                }
                                e_re[s] = cs;
                                e_im[s] = sn;
                            } else {
                                PhaseOps<R>::exact(rec, xq0, xq1, xq2, x0, x1, x2, &sn, &cs);
                            }
                            zre = cs; zim = sn;
                            if constexpr (ADIAG) {
                                R q;
                                if constexpr (WHT) q = qw[s & 3];
                                else q = qd + xs(3) * qc[0] + xs(5) * qc[1] + xs(6) * qc[2];
                                const R T = texp<R>(-q);
                                zre *= T; zim *= T;
                            } else if constexpr (ANISO) {
                                const R q = adp[0] * m6[0] + adp[1] * m6[1] + adp[2] * m6[2] + adp[3] * m6[3] +
                                            adp[4] * m6[4] + adp[5] * m6[5];
                                const R T = texp<R>(-q);
                                zre *= T; zim *= T;
                            }
                            if constexpr (INV) {
                                zT_re[s < NR / 2 ? s : 0] = zre;
                                zT_im[s < NR / 2 ? s : 0] = zim;
                            }
                        }
                        R fre, fim;
                        R A0 = 0, A1 = 0, A2 = 0, A3 = 0, A4 = 0;
                        const R *y = rec.y;
                        if constexpr (TABLE) {
                            // the table holds n_hkl_pad rows (zero past the last reflection), columns in the
                            // engine's atom order, each column's operation values contiguous (consecutive lanes
                            // read consecutive columns)
                            if constexpr (TAB_REG) {
                                const float2 tv = __fadd2_rn(cur[j * NR + s], make_float2(anre, anim));
                                fre = tv.x; fim = tv.y;
                            } else if constexpr (F32) {
                                const float2 tv = reinterpret_cast<const float2 *>(st + SL.tab)[
                                    ((size_t)hl * kTileAtoms + tid) * nS + s];
                                fre = tv.x + anre; fim = tv.y + anim;
                            } else {
                                const int col = a + (a >= S.table_split ? S.table_shift : 0);
                                const size_t ti = ((size_t)(h0 + hl) * S.table_stride + (have ? col : 0)) * nS + s;
                                // an FP32-only table is read widened
                                double2 tv;
                                if (S.table_d) {
                                    tv = S.table_d[ti];
                                } else {
                                    const float2 t1 = S.table_f[ti];
                                    tv = make_double2(t1.x, t1.y);
                                }
                                fre = tv.x + anre; fim = tv.y + anim;
                            }
                        } else if constexpr (DIAG && WHT) {
                            fre = fwr[s & 3];
                            fim = fwi[s & 3];
                        } else if constexpr (DIAG) {
                            // fsph rides in the class-0 sums (sign +1 for every operation)
                            if constexpr (F32) {
                                fre = Ec[0] + G.f[s][3] * Ec[1] + G.f[s][6] * Ec[2] + G.f[s][5] * Ec[3];
                                fim = fsim + G.f[s][2] * Oc[0] + G.f[s][4] * Oc[1] + G.f[s][1] * Oc[2] +
                                      G.f[s][7] * Oc[3];
                            } else {
                                fre = Ec[0] + G.d[s][3] * Ec[1] + G.d[s][6] * Ec[2] + G.d[s][5] * Ec[3];
                                fim = fsim + G.d[s][2] * Oc[0] + G.d[s][4] * Oc[1] + G.d[s][1] * Oc[2] +
                                      G.d[s][7] * Oc[3];
                            }
                        } else if constexpr (HC) {
                            A0 = pg[0] * y[0];
                            A1 = pg[1] * y[1] + pg[2] * y[2] + pg[3] * y[3];
                            A2 = pg[4] * y[4] + pg[5] * y[5] + pg[6] * y[6] + pg[7] * y[7] + pg[8] * y[8];
                            if (high_l) {
                                A3 = pg[9] * y[9] + pg[10] * y[10] + pg[11] * y[11] + pg[12] * y[12] +
                                     pg[13] * y[13] + pg[14] * y[14] + pg[15] * y[15];
                                A4 = pg[16] * y[16] + pg[17] * y[17] + pg[18] * y[18] + pg[19] * y[19] +
                                     pg[20] * y[20] + pg[21] * y[21] + pg[22] * y[22] + pg[23] * y[23] +
                                     pg[24] * y[24];
                            }
                            fre = fsre + r0 * A0 + r2 * A2 + r4 * A4;
                            fim = fsim + r1 * A1 + r3 * A3;
                        } else {
                            fre = fsre;
                            fim = fsim;
                        }
                        const R ure = fre * zre - fim * zim;
                        const R uim = fre * zim + fim * zre;
                        if constexpr (WHT) {
                            // every sum over the coset's operations follows from these at its end (wht_end)
                            ur4[s & 3] = ure;
                            ui4[s & 3] = uim;
                        } else if (NSC > 0 && s == 0) {  // compile-time with a compiled operation count
                            Ure = ure; Uim = uim;
                        } else {
                            Ure += ure; Uim += uim;
                        }
                        if constexpr (WHT) {
                        } else if constexpr (XDIAG) {
                            // signed sums: x y z -> slots 0 1 2 (classes 1 2 4), xy xz yz -> 3 4 5 (3 5 6);
                            // the coset's first operation has every sign +1 (s is a compile-time index here)
                            const bool first = s % (CS > 0 ? CS : 1) == 0;
                            constexpr int cls[6] = {1, 2, 4, 3, 5, 6};
#pragma unroll
                            for (int q = 0; q < NSG; q++) {
                                if (first) {
                                    Sre[q] = ure; Sim[q] = uim;
                                } else {
                                    Sre[q] += xs(cls[q]) * ure; Sim[q] += xs(cls[q]) * uim;
                                }
                            }
                            if constexpr (ADIAG) { Ucre += ure; Ucim += uim; }
                        } else {
                            Xre[0] += h0f * ure; Xim[0] += h0f * uim;
                            Xre[1] += h1f * ure; Xim[1] += h1f * uim;
                            Xre[2] += h2f * ure; Xim[2] += h2f * uim;
                            if constexpr (ANISO) {
#pragma unroll
                                for (int q = 0; q < 6; q++) { Are[q] -= m6[q] * ure; Aim[q] -= m6[q] * uim; }
                            }
                        }
                        if constexpr (MP) {
                            // q_l = Re(g i^l rr_l z): even l rs_l Re(gz), odd l -rs_l Im(gz)
                            const R wre = gre * zre - gim * zim, wim = gre * zim + gim * zre;
                            if constexpr (DIAG) {
                                // everything else of the multipole adjoint follows from these sums
                                // once per coset (flush_slots)
                                const auto sg = [&](int c) -> R {
                                    if constexpr (F32) return G.f[s][c]; else return G.d[s][c];
                                };
                                if constexpr (WHT) {
                                    wr4[s & 3] = wre;
                                    wi4[s & 3] = wim;
                                } else {
                                We[0] += wre; We[1] += sg(3) * wre; We[2] += sg(6) * wre; We[3] += sg(5) * wre;
                                Wo[0] += sg(2) * wim; Wo[1] += sg(4) * wim; Wo[2] += sg(1) * wim; Wo[3] += sg(7) * wim;
                                }
                            } else {
                                const R *dr = sTrm + (size_t)(lt * ht + hl) * 8;
                                Ere += zre; Eim += zim;
                                const R q0 = r0 * wre, q1 = -r1 * wim, q2 = r2 * wre, q3 = -r3 * wim, q4 = r4 * wre;
                                part[CH_PLM] += q0 * y[0];
#pragma unroll
                                for (int q = 1; q < 4; q++) part[CH_PLM + q] += q1 * y[q];
#pragma unroll
                                for (int q = 4; q < 9; q++) part[CH_PLM + q] += q2 * y[q];
#pragma unroll
                                for (int q = 9; q < 16; q++) part[CH_PLM + q] += q3 * y[q];
#pragma unroll
                                for (int q = 16; q < 25; q++) part[CH_PLM + q] += q4 * y[q];
                                const R dre = dr[2] * A0 + dr[4] * A2 + dr[6] * A4;
                                const R dim = dr[3] * A1 + dr[5] * A3;
                                Kre += dre * zre - dim * zim;
                                Kim += dre * zim + dim * zre;
                            }
                        }
                    };
                    if constexpr (NSC > 0) {
#pragma unroll
                        for (int s = 0; s < NSC; s++) {
                            if constexpr (CS > 0) {
                                if (s % CS == 0) {
                                    if (s > 0) {
                                        wht_end();
                                        flush_slots(recs[s - CS].y, sTrm + (size_t)(lt * ht + hl) * 8);
                                        adp_coset_end();
                                    }
                                    class_sums(recs[s].y);
                                    mp_coset_begin(recs[s].y, sTrm + (size_t)(lt * ht + hl) * 8);
                                    forward_wht();
                                    adp_coset_begin(recs[s]);
                                }
                            }
                            term(s);
                        }
                        if constexpr (CS > 0) {
                            wht_end();
                            flush_slots(recs[NSC - CS].y, sTrm + (size_t)(lt * ht + hl) * 8);
                            adp_coset_end();
                        }
                    } else {
#pragma unroll 1
                        for (int s = 0; s < nS; s++) term(s);
                    }
                    // the isotropic factor rides in the weights: w T for F, g T (gre, gim) for the adjoint
                    const R wT = w * Tiso;
                    if constexpr (ROLL_J) {
                        const R fv0 = wT * Ure, fv1 = wT * Uim;
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            if (q == j) { Fv[2 * q] = fv0; Fv[2 * q + 1] = fv1; }
                    } else {
                        Fv[2 * j] = wT * Ure;
                        Fv[2 * j + 1] = wT * Uim;
                    }
                    R gU;  // Re(g T U)
                    if constexpr (WHT) gU = gUc; else gU = gre * Ure - gim * Uim;
                    part[CH_OCC] += gU;
                    if constexpr (!ANISO) {
                        part[CH_ADP] -= sH2[hl] * gU;
                    } else if constexpr (!WHT) {
#pragma unroll
                        for (int q = 0; q < 6; q++) part[CH_ADP + q] += gre * Are[q] - gim * Aim[q];
                    }
                    if constexpr (!WHT)
#pragma unroll
                        for (int q = 0; q < 3; q++) part[CH_XYZ + q] -= gre * Xim[q] + gim * Xre[q];  // -Im(g T X)
                    if constexpr (MP && !DIAG) {
                        const R *dr = sTrm + (size_t)(lt * ht + hl) * 8;
                        const R gE = gre * Ere - gim * Eim;
                        part[CH_PV] += dr[0] * gE;
                        part[CH_KAPPA] += dr[1] * gE;
                        part[CH_KAPPA_P] += gre * Kre - gim * Kim;
                    }
                }
            };
            if constexpr (ROLL_J) {
#pragma unroll 1
                for (int j = 0; j < 4; j++) reflection(j);
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) reflection(j);
            }
            // butterfly reduce-scatter of the group's 8 values over the warp:
            // value index 4*bit4 + 2*bit3 + bit2 of the lane ends summed in lanes with bits 1,0 = 0
            const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
            R v4[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const R keep = b4 ? Fv[q + 4] : Fv[q], send = b4 ? Fv[q] : Fv[q + 4];
                v4[q] = keep + shfl_xor<R>(send, 16);
            }
            R v2[2];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const R keep = b3 ? v4[q + 2] : v4[q], send = b3 ? v4[q] : v4[q + 2];
                v2[q] = keep + shfl_xor<R>(send, 8);
            }
            R v1 = (b2 ? v2[1] : v2[0]) + shfl_xor<R>(b2 ? v2[0] : v2[1], 4);
            v1 += shfl_xor<R>(v1, 2);
            v1 += shfl_xor<R>(v1, 1);
            if ((lane & 3) == 0) {
                const int idx = lane >> 2;  // 0..7 = 4*b4 + 2*b3 + b2
                R *dst = reinterpret_cast<R *>(&sF[warp * ht + g0 + (idx >> 1)]);
                dst[idx & 1] = v1;
            }
        };
        if constexpr (TAB_REG) {
            // the group's form factors (loaded one group ahead) move to `tab_a`; `group` loads the next group's
            // into `tab_b`.  (Two buffers taking turns without the copy spill the anisotropic kernels under the
            // four-block register cap.)
#pragma unroll 1
            for (int g0 = 0; g0 < ht; g0 += 4) {
#pragma unroll
                for (int q = 0; q < kTabN; q++) tab_a[q] = tab_b[q];
                group(g0, tab_a, tab_b);
            }
        } else {
#pragma unroll 1
            for (int g0 = 0; g0 < ht; g0 += 4) group(g0, tab_a, tab_b);
        }
        // fold the partial sums into the Kahan totals (each thread its own column;
        // isotropic tiles use one ADP channel of six)
        if (GRAD && ((k + 1) % fold == 0 || h0 + ht >= h_end)) {
#pragma unroll
            for (int q = 0; q < NT; q++) {
            if (!ANISO && q > CH_ADP && q < CH_OCC) continue;
            R sum = sTot[q * kTileAtoms + tid], comp = sCmp[q * kTileAtoms + tid];
            const R yv = part[q] - comp;
            const R tv = sum + yv;
            comp = (tv - sum) - yv;
            sTot[q * kTileAtoms + tid] = tv;
            sCmp[q * kTileAtoms + tid] = comp;
            part[q] = R(0);
            }
        }
        __syncthreads();
        for (int i = tid; i < ht; i += blockDim.x) {
            R sre = 0, sim = 0;
#pragma unroll
            for (int wp = 0; wp < kWarps; wp++) {
            const R2 v = sF[wp * ht + i];
            sre += v.x;
            sim += v.y;
            }
            atomicAdd(&C.f_acc[h0 + i].x, (double)sre);
            atomicAdd(&C.f_acc[h0 + i].y, (double)sim);
        }
        __syncthreads();
    }
    if (GRAD && active) {
        double *G = C.g_acc + (size_t)a * kNch;
        auto total = [&](int q) {
            return (double)sTot[q * kTileAtoms + tid] - (double)sCmp[q * kTileAtoms + tid];
        };
#pragma unroll
        for (int q = 0; q < 3; q++) atomicAdd(G + CH_XYZ + q, total(CH_XYZ + q));
        if (ANISO) {
#pragma unroll
            for (int q = 0; q < 6; q++) atomicAdd(G + CH_ADP + q, total(CH_ADP + q));
        } else if (has_adp) {
            atomicAdd(G + CH_ADP, total(CH_ADP));
        }
        atomicAdd(G + CH_OCC, total(CH_OCC));
        if constexpr (MP) {
#pragma unroll
            for (int q = CH_PV; q < NT; q++) atomicAdd(G + q, total(q));
        }
    }
}

// one structure: block (tile, reflection chunk)
template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS = 0, bool GRAD = true, bool INV = false,
          int PAT = 0>
__global__ void __launch_bounds__(kTileAtoms)
sf_grad_kernel3(DevStructure S, CallBuffers C, SfLaunch L, SignTable G)
{
    sf_grad_body<R, MODEL, MP, ANISO, NSC, CS, GRAD, INV, PAT>(S, C, L, G, blockIdx.x, blockIdx.y);
}

// the same with at least three blocks per SM: a register cap (168) for the FP32 multipole-adjoint kernels, which
// the compiler otherwise gives about 220 registers (two blocks per SM); the autotuner times both and keeps the
// faster (it trades a few spills for half again as many warps)
template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS = 0, bool GRAD = true, bool INV = false,
          int PAT = 0>
__global__ void __launch_bounds__(kTileAtoms, 3)
sf_grad_kernel3_occ3(DevStructure S, CallBuffers C, SfLaunch L, SignTable G)
{
    sf_grad_body<R, MODEL, MP, ANISO, NSC, CS, GRAD, INV, PAT>(S, C, L, G, blockIdx.x, blockIdx.y);
}

// the same with at least four blocks per SM: the tabulated model with up to
// four compiled operations (HBM streaming: occupancy over registers).  The
// other kernels keep the compiler's own register choice, which an explicit
// minimum of one block would change.
template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS = 0, bool GRAD = true, bool INV = false,
          int PAT = 0>
__global__ void __launch_bounds__(kTileAtoms, 4)
sf_grad_kernel3_occ4(DevStructure S, CallBuffers C, SfLaunch L, SignTable G)
{
    sf_grad_body<R, MODEL, MP, ANISO, NSC, CS, GRAD, INV, PAT>(S, C, L, G, blockIdx.x, blockIdx.y);
}

// many structures of one kernel shape (and one sign table) in one launch: the
// block's item is the last with block_begin <= blockIdx.x
template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS, bool INV, int PAT = 0>
__device__ __forceinline__ void sf_grad_batch_body(const SfBatch &B, const SignTable &G)
{
    const int b = blockIdx.x;
    int lo = 0, hi = B.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B.block_begin[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const SfBatchItem &it = B.item[lo];
    const int lb = b - B.block_begin[lo];
    sf_grad_body<R, MODEL, MP, ANISO, NSC, CS, true, INV, PAT>(it.S, it.C, it.L, G, lb % it.n_tiles,
                                                               lb / it.n_tiles);
}

template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS = 0, bool INV = false, int PAT = 0>
__global__ void __launch_bounds__(kTileAtoms)
sf_grad_batch3(const __grid_constant__ SfBatch B, const __grid_constant__ SignTable G)
{
    sf_grad_batch_body<R, MODEL, MP, ANISO, NSC, CS, INV, PAT>(B, G);
}

template <typename R, int MODEL, bool MP, bool ANISO, int NSC, int CS = 0, bool INV = false, int PAT = 0>
__global__ void __launch_bounds__(kTileAtoms, 4)
sf_grad_batch3_occ4(const __grid_constant__ SfBatch B, const __grid_constant__ SignTable G)
{
    sf_grad_batch_body<R, MODEL, MP, ANISO, NSC, CS, INV, PAT>(B, G);
}

// kernels that take the four-block minimum: FP32 tabulated, form factors in registers
template <typename R, int MODEL, int NSC>
constexpr bool occ4_kernel() { return sizeof(R) == 4 && MODEL == MODEL_TABLE && NSC > 0 && NSC <= 4; }

}  // namespace dsf
