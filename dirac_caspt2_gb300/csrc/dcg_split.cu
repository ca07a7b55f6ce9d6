// Split-precision complex GEMM on the 5th-generation tensor cores (tcgen05, TMEM), the
// DCG_PREC_SPLIT path of the 4-index transformation.
//
// C (M x N complex) = A (M x K complex) * op(B) (K x N complex), with A large (a slice of an
// integral class) and B small (an orbital rotation).  Written from the error-free splitting
// idea of Ozaki, Ogita, Oishi & Rump (Numer. Algorithms 59 (2012) 95) on BF16 tensor cores:
//
//   * complex -> real: A' = [Re a, Im a] interleaved along K (the complex memory layout), and
//     B' (2K x 2N) with B'(2k,2j) = Re b, B'(2k+1,2j) = -Im b, B'(2k,2j+1) = Im b,
//     B'(2k+1,2j+1) = Re b, so that C' = A' B' is C with Re and Im interleaved;
//   * each row of A' is scaled by 2^-e (e: exponent of its largest entry) and each column pair
//     of B' by 2^-f; the scaled values are cut into SPLIT_S slices of SPLIT_BITS bits,
//     x = sum_p sigma_p 2^(-7p), sigma_p integers (|sigma_1| <= 128, |sigma_p| <= 64), each
//     stored exactly in BF16 already multiplied by 2^(-7(p-1));
//   * the products A_p B_q with p + q <= SPLIT_S + 1 (15 of 25) are accumulated in FP32 in four
//     TMEM accumulators by weight p+q = 2, 3, 4 and >= 5.  The first three stay exact (integer
//     partial sums below 2^24 for K' <= 1024 real); the last one carries only 2^-21-relative
//     terms, so its rounding is ~2^-45 of the result;
//   * the epilogue adds the accumulators (the exact pair kept exact by an FP32 TwoSum) and applies
//     2^(e+f-14) through the exponent field.
// The result carries ~2^-36 of max|row of A| * max|column of B| per term.
//
// Data movement: the slicing pre-pass writes both operands directly in the tcgen05 canonical
// K-major, no-swizzle layout, tile by tile (128 rows x 16 real K = 4 KB per slice), so every
// pipeline stage is filled by plain bulk copies (cp.async.bulk) completing on an mbarrier.
// One warp produces, one thread issues the 15 MMAs per K-step, four warps read TMEM back.
// Every wait is bounded; a wait that runs out sets an error flag and the kernel unwinds.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "dcg_common.cuh"

namespace dcg {

constexpr int SPLIT_S = 5;          // slices per operand
constexpr int SPLIT_BITS = 7;       // bits per slice
constexpr int SP_TM = 128;          // CTA rows (TMEM lanes)
constexpr int SP_TN = 128;          // CTA real output columns (per accumulator)
constexpr int SP_TK = 16;           // real K per MMA
constexpr int SP_KMAX = 1024;       // real K per launch (exact FP32 groups)
constexpr int SP_STAGES = 4;
constexpr int SP_TILE_BYTES = SP_TM * SP_TK * 2;                       // 4096
constexpr int SP_STAGE_BYTES = 2 * SPLIT_S * SP_TILE_BYTES;            // A and B slices: 40 KB
constexpr int SP_SMEM = SP_STAGES * SP_STAGE_BYTES + 1024;             // + alignment
constexpr int SP_THREADS = 192;     // warps 0-3 epilogue, 4 producer, 5 MMA issuer
constexpr uint64_t SP_WAIT_NS = 2000000000ull;

// Byte offset of element (r, kk) inside a 128 x 16 K-major tile: 8 x 8 core matrices of
// 128 B (8 rows of 16 B), the two K-adjacent core matrices SP_KGRP bytes apart, the sixteen
// 8-row groups SP_MGRP bytes apart.  The MMA descriptors carry these two strides.
constexpr int SP_KGRP = 128, SP_MGRP = 256;
__host__ __device__ __forceinline__ int sp_tile_off(int r, int kk) {
    return (r >> 3) * SP_MGRP + (kk >> 3) * SP_KGRP + (r & 7) * 16 + (kk & 7) * 2;
}

// ------------------------------------------------------------------------- slicing pre-passes
// All slicing is integer arithmetic on the IEEE-754 bit pattern (GB300 retires about two FP64
// FMAs per clock per SM, its integer and FP32 pipes many more).

// exponent e with |x| <= 2^e for the largest |x| of a row (0 for an all-zero row); the
// argument is the largest (sign-cleared) bit pattern, which orders like the magnitude
__device__ __forceinline__ int sp_exponent_bits(long long mb) {
    const int ex = (int)((mb >> 52) & 0x7FF);
    return ex == 0 ? 0 : ex - 1022;   // normal: |x| < 2^(ex-1022); subnormal rows count as zero
}
__device__ __forceinline__ long long sp_absbits(double x) { return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll; }

// The S pre-scaled slices of x 2^-e (|x| <= 2^e): X = round(x 2^(7S-e)) as a signed integer,
// cut into balanced base-128 digits d_0..d_{S-1} (|d_0| <= 128, others <= 64);
// out[p] = d_p 2^(-7p), so that x 2^-e = 2^-7 sum_p out[p] up to 2^-(7S+1).  S = 5 for the
// transformation products, S = 7 for the products that feed the metric's inverse.
template <int S>
__device__ __forceinline__ void sp_slices(double x, int e, __nv_bfloat16 out[S]) {
    const long long bits = __double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    long long X = 0;
    if (ex != 0) {
        const long long mant = (bits & ((1ll << 52) - 1)) | (1ll << 52);   // |x| = mant 2^(ex-1075)
        const int sh = ex - 1075 + SPLIT_BITS * S - e;
        if (sh >= 0) X = mant << sh;                                        // only when |x| ~ 2^e and tiny mantissa
        else if (sh > -54) X = (mant + (1ll << (-sh - 1))) >> (-sh);
        if (bits < 0) X = -X;
    }
#pragma unroll
    for (int p = 0; p < S - 1; p++) {
        const int sft = SPLIT_BITS * (S - 1 - p);
        const long long d = (X + (1ll << (sft - 1))) >> sft;
        X -= d << sft;
        out[p] = __float2bfloat16_rn(__int2float_rn((int)d) * __int_as_float((127 - SPLIT_BITS * p) << 23));
    }
    out[S - 1] = __float2bfloat16_rn(__int2float_rn((int)X) * __int_as_float((127 - SPLIT_BITS * (S - 1)) << 23));
}

// Row exponents of the large operand: element (i, k) of batch z at A[z*sb + i*si + k*sk].
// rows_contig (si == 1): one thread per row.  Otherwise one warp per row (k contiguous).
__global__ void sp_rowexp_kernel(int M, int K, const cplx *__restrict__ A, int64_t si, int64_t sk, int64_t sb,
                                 int rows_contig, int *eexp) {
    const int z = blockIdx.y;
    if (rows_contig) {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= M) return;
        const cplx *a = A + (int64_t)z * sb + (int64_t)i * si;
        long long mb = 0;
        for (int k = 0; k < K; k++) {
            const cplx v = a[(int64_t)k * sk];
            mb = max(mb, max(sp_absbits(v.x), sp_absbits(v.y)));
        }
        eexp[(int64_t)z * M + i] = sp_exponent_bits(mb);
    } else {
        const int lane = threadIdx.x & 31;
        const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
        if (i >= M) return;
        const cplx *a = A + (int64_t)z * sb + (int64_t)i * si;
        long long mb = 0;
        for (int k = lane; k < K; k += 32) {
            const cplx v = a[(int64_t)k * sk];
            mb = max(mb, max(sp_absbits(v.x), sp_absbits(v.y)));
        }
        for (int o = 16; o > 0; o >>= 1) mb = max(mb, __shfl_down_sync(0xffffffffu, mb, o));
        if (lane == 0) eexp[(int64_t)z * M + i] = sp_exponent_bits(mb);
    }
}

// The same for few contiguous rows (si == 1, M small, K long: the Gram factor of the A/C blocks):
// a block takes 32 rows and 32 strands of k, so each warp reads 32 adjacent rows at one k and a
// thread scans K/32 entries instead of K; the strands' maxima meet in shared memory.
__global__ void __launch_bounds__(1024) sp_rowexp_tile_kernel(int M, int K, const cplx *__restrict__ A, int64_t sk,
                                                              int64_t sb, int *eexp) {
    __shared__ long long red[32][33];
    const int z = blockIdx.y;
    const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int i = blockIdx.x * 32 + r;
    long long mb = 0;
    if (i < M) {
        const cplx *a = A + (int64_t)z * sb + i;
        for (int k = g; k < K; k += 32) {
            const cplx v = a[(int64_t)k * sk];
            mb = max(mb, max(sp_absbits(v.x), sp_absbits(v.y)));
        }
    }
    red[g][r] = mb;
    __syncthreads();
    if (g == 0 && i < M) {
        long long m = 0;
        for (int q = 0; q < 32; q++) m = max(m, red[q][r]);
        eexp[(int64_t)z * M + i] = sp_exponent_bits(m);
    }
}

// Row exponents through whichever kernel suits the shape.
static void launch_rowexp(Context &c, int M, int K, int batch, const cplx *A, int64_t a_si, int64_t a_sk, int64_t a_sb,
                          int *eexp) {
    if (a_si == 1 && M < 32768 && K >= 64) {
        sp_rowexp_tile_kernel<<<dim3((unsigned)((M + 31) / 32), batch), 1024, 0, c.stream>>>(M, K, A, a_sk, a_sb, eexp);
    } else if (a_si == 1) {
        dim3 g(grid1d(M, 256), batch);
        sp_rowexp_kernel<<<g, 256, 0, c.stream>>>(M, K, A, a_si, a_sk, a_sb, 1, eexp);
    } else {
        dim3 g(grid1d((int64_t)M * 32, 256), batch);
        sp_rowexp_kernel<<<g, 256, 0, c.stream>>>(M, K, A, a_si, a_sk, a_sb, 0, eexp);
    }
    DCG_LAUNCHED(c);
}

// A slices in tiles: tile (p, z, rb, ks) at ((p*nz + z)*nrb + rb)*nks + ks, 4 KB each.
// One thread per (row, group of 4 complex k) writes one 16-byte core-matrix row per slice.
template <int S>
__global__ void sp_slice_a_kernel(int M, int K, const cplx *__restrict__ A, int64_t si, int64_t sk, int64_t sb,
                                  const int *__restrict__ eexp, int nz, int nrb, int nks, __nv_bfloat16 *As) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    const int ng = nks * (SP_TK / 8);              // 8-real groups along K'
    const int64_t rows = (int64_t)nrb * SP_TM;
    if (idx >= rows * ng) return;
    const int i = (int)(idx % rows), g = (int)(idx / rows);
    __align__(16) __nv_bfloat16 sl[S][8];
    if (i < M) {
        const int e = eexp[(int64_t)z * M + i];
        const cplx *a = A + (int64_t)z * sb + (int64_t)i * si;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int k = g * 4 + c;
            cplx v = mk(0.0, 0.0);
            if (k < K) v = a[(int64_t)k * sk];
            __nv_bfloat16 re[S], im[S];
            sp_slices<S>(v.x, e, re);
            sp_slices<S>(v.y, e, im);
#pragma unroll
            for (int p = 0; p < S; p++) {
                sl[p][2 * c] = re[p];
                sl[p][2 * c + 1] = im[p];
            }
        }
    } else {
#pragma unroll
        for (int p = 0; p < S; p++)
#pragma unroll
            for (int q = 0; q < 8; q++) sl[p][q] = __float2bfloat16_rn(0.0f);
    }
    const int rb = i / SP_TM, r = i % SP_TM;
    const int ks = g / (SP_TK / 8), kk = (g % (SP_TK / 8)) * 8;
    for (int p = 0; p < S; p++) {
        const int64_t tile = (((int64_t)p * nz + z) * nrb + rb) * nks + ks;
        char *dst = reinterpret_cast<char *>(As) + tile * SP_TILE_BYTES + sp_tile_off(r, kk);
        *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(sl[p]);
    }
}

// B' slices (N'-major tiles: tile (q, nb, ks) at (q*nnb + nb)*nks + ks) and column exponents.
// op(B)(k, j) = B[k + j ldb], or B[j + k ldb] when opb & 2 (B stored transposed), conjugated
// when opb & 1.  One block per complex column j.
template <int S>
__global__ void sp_slice_b_kernel(int K, int N, const cplx *__restrict__ B, int64_t ldb, int opb, int nnb, int nks,
                                  __nv_bfloat16 *Bs, int *fexp) {
    __shared__ long long red[32];
    const int j = blockIdx.x;
    long long mb = 0;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const cplx v = (opb & 2) ? B[j + (int64_t)k * ldb] : B[k + (int64_t)j * ldb];
        mb = max(mb, max(sp_absbits(v.x), sp_absbits(v.y)));
    }
    for (int o = 16; o > 0; o >>= 1) mb = max(mb, __shfl_down_sync(0xffffffffu, mb, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mb;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long m = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = max(m, red[w]);
        red[0] = m;
    }
    __syncthreads();
    const int f = sp_exponent_bits(red[0]);
    if (threadIdx.x == 0) fexp[j] = f;
    const int kp = nks * SP_TK;   // real K, padded
    for (int kr = threadIdx.x; kr < kp; kr += blockDim.x) {
        const int k = kr >> 1, part = kr & 1;   // real row 2k (Re) or 2k+1 (Im) of B'
        cplx v = mk(0.0, 0.0);
        if (k < K) {
            v = (opb & 2) ? B[j + (int64_t)k * ldb] : B[k + (int64_t)j * ldb];
            if (opb & 1) v = cconj(v);
        }
        // column 2j: (Re, -Im) down the real rows; column 2j+1: (Im, Re)
        const double c0 = part == 0 ? v.x : -v.y;
        const double c1 = part == 0 ? v.y : v.x;
        __nv_bfloat16 s0[S], s1[S];
        sp_slices<S>(c0, f, s0);
        sp_slices<S>(c1, f, s1);
        const int ks = kr / SP_TK, kk = kr % SP_TK;
        for (int col = 0; col < 2; col++) {
            const int jr = 2 * j + col;
            const int nb = jr / SP_TN, r = jr % SP_TN;
            for (int q = 0; q < S; q++) {
                const int64_t tile = ((int64_t)q * nnb + nb) * nks + ks;
                __nv_bfloat16 *dst = reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(Bs) +
                                                                       tile * SP_TILE_BYTES + sp_tile_off(r, kk));
                *dst = col == 0 ? s0[q] : s1[q];
            }
        }
    }
}

// ------------------------------------------------------------------------- tcgen05 GEMM
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t sp_now() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// bounded wait; false (and *err set) when limit_ns runs out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = sp_now();
    while (!mbar_try_wait(bar, parity)) {
        if (*(volatile int *)err) return false;
        if (sp_now() - t0 > limit_ns) {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(64);
    }
    return true;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), version 1, no swizzle
__device__ __forceinline__ uint64_t sp_desc(const void *p, int lbo, int sbo) {
    const uint64_t a = (smem_u32(p) >> 4) & 0x3FFFull;
    return a | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// instruction descriptor: kind::f16, D f32, A/B bf16, both K-major, N = SP_TN, M = SP_TM
constexpr uint32_t SP_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(SP_TN >> 3) << 17) |
                              ((uint32_t)(SP_TM >> 4) << 24);

__device__ __forceinline__ void umma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(SP_IDESC), "r"(acc));
}
// instruction descriptor of the persistent kernel's 128 x 64 products
constexpr int SPP_TN = 64;
constexpr uint32_t SPP_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(SPP_TN >> 3) << 17) |
                               ((uint32_t)(SP_TM >> 4) << 24);

__device__ __forceinline__ void umma_f16_n64(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(SPP_IDESC), "r"(acc));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// wait used while shutting down after an error: bounded by time only
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity) {
    const uint64_t t0 = sp_now();
    while (!mbar_try_wait(bar, parity)) {
        if (sp_now() - t0 > SP_WAIT_NS) return;
        __nanosleep(64);
    }
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

#define SP_LD32(taddr, r)                                                                                        \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15," \
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                      \
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),        \
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),    \
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), \
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), \
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])                                          \
                 : "r"(taddr))

struct SplitArgs {
    const __nv_bfloat16 *As, *Bs;
    const int *eexp, *fexp;
    cplx *C;
    int64_t c_si, c_sj, c_sb;
    int M, N, nz, nrb, nnb, nks;
    int lbo, sbo;     // descriptor leading / stride byte offsets
    int accumulate;   // C += result
    int order;        // CTA raster: 0 column blocks of a row block adjacent, 1 row blocks of a column block
    int *err;
    uint64_t wait_ns;   // limit of the pipeline waits (SP_WAIT_NS unless a test shortens it)
};

// g0 + g1 + g2 + g3 (FP32 bit patterns) as a double: TwoSum (Knuth) keeps g0 + g1 exact as
// s + t, then g2 + g3 are added to t in FP32.
__device__ __forceinline__ double recombine(uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
    const float g0 = __uint_as_float(b0), g1 = __uint_as_float(b1);
    const float s = __fadd_rn(g0, g1);
    const float bb = __fsub_rn(s, g0);
    const float t = __fadd_rn(__fsub_rn(g0, __fsub_rn(s, bb)), __fsub_rn(g1, bb));
    const float lo = __fadd_rn(t, __fadd_rn(__uint_as_float(b2), __uint_as_float(b3)));
    return (double)s + (double)lo;
}

// v 2^sc: an integer add to the exponent field when v and the result are normal numbers.
__device__ __forceinline__ double scale_pow2(double v, int sc) {
    const long long bits = __double_as_longlong(v);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (v != 0.0 && ex > 0 && ex + sc > 0 && ex + sc < 2047) return __longlong_as_double(bits + ((long long)sc << 52));
    return v * ldexp(1.0, sc);
}

__global__ void __launch_bounds__(SP_THREADS, 1) sp_gemm_kernel(SplitArgs a) {
    extern __shared__ __align__(1024) unsigned char sp_raw[];
    __shared__ __align__(8) uint64_t bar_full[SP_STAGES], bar_empty[SP_STAGES], bar_done;
    __shared__ uint32_t s_tmem;
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(sp_raw) + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // linear (row block, column block) index: order 0 keeps the column blocks of a row block
    // adjacent (the CTAs sharing an A tile run together and find it in L2), order 1 the row
    // blocks of a column block (sharing a B tile); the autotuner picks per shape
    const int rb = a.order ? (int)(blockIdx.x % (unsigned)a.nrb) : (int)(blockIdx.x / (unsigned)a.nnb);
    const int nb = a.order ? (int)(blockIdx.x / (unsigned)a.nrb) : (int)(blockIdx.x % (unsigned)a.nnb);
    const int z = blockIdx.z;

    if (threadIdx.x == 0) {
        for (int s = 0; s < SP_STAGES; s++) {
            mbar_init(&bar_full[s], 1);
            mbar_init(&bar_empty[s], 1);
        }
        mbar_init(&bar_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {   // 4 accumulators x SP_TN columns = 512 TMEM columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(4 * SP_TN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;
    const int nks = a.nks;
    int issued = 0;   // producer: stages whose copies were issued

    if (warp == 4) {
        if (lane == 0) {   // producer: 2 x SPLIT_S bulk copies of 4 KB per stage
            for (int ks = 0; ks < nks; ks++) {
                const int s = ks % SP_STAGES;
                if (ks >= SP_STAGES && !mbar_wait(&bar_empty[s], ((ks / SP_STAGES) - 1) & 1, a.err, a.wait_ns)) break;
                issued = ks + 1;
                unsigned char *st = smem + s * SP_STAGE_BYTES;
                mbar_expect_tx(&bar_full[s], SP_STAGE_BYTES);
                for (int p = 0; p < SPLIT_S; p++) {
                    const int64_t ta = (((int64_t)p * a.nz + z) * a.nrb + rb) * nks + ks;
                    bulk_g2s(st + p * SP_TILE_BYTES, reinterpret_cast<const char *>(a.As) + ta * SP_TILE_BYTES,
                             SP_TILE_BYTES, &bar_full[s]);
                    const int64_t tb = ((int64_t)p * a.nnb + nb) * nks + ks;
                    bulk_g2s(st + (SPLIT_S + p) * SP_TILE_BYTES, reinterpret_cast<const char *>(a.Bs) + tb * SP_TILE_BYTES,
                             SP_TILE_BYTES, &bar_full[s]);
                }
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {   // MMA issuer
            bool ok = true;
            for (int ks = 0; ks < nks && ok; ks++) {
                const int s = ks % SP_STAGES;
                if (!mbar_wait(&bar_full[s], (ks / SP_STAGES) & 1, a.err, a.wait_ns)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const unsigned char *st = smem + s * SP_STAGE_BYTES;
                uint64_t da[SPLIT_S], db[SPLIT_S];
#pragma unroll
                for (int p = 0; p < SPLIT_S; p++) {
                    da[p] = sp_desc(st + p * SP_TILE_BYTES, a.lbo, a.sbo);
                    db[p] = sp_desc(st + (SPLIT_S + p) * SP_TILE_BYTES, a.lbo, a.sbo);
                }
                const uint32_t first = ks > 0 ? 1u : 0u;
                // weight 2
                umma_f16(tmem + 0 * SP_TN, da[0], db[0], first);
                // weight 3
                umma_f16(tmem + 1 * SP_TN, da[0], db[1], first);
                umma_f16(tmem + 1 * SP_TN, da[1], db[0], 1u);
                // weight 4
                umma_f16(tmem + 2 * SP_TN, da[0], db[2], first);
                umma_f16(tmem + 2 * SP_TN, da[1], db[1], 1u);
                umma_f16(tmem + 2 * SP_TN, da[2], db[0], 1u);
                // weights 5 and 6
                umma_f16(tmem + 3 * SP_TN, da[0], db[3], first);
                umma_f16(tmem + 3 * SP_TN, da[1], db[2], 1u);
                umma_f16(tmem + 3 * SP_TN, da[2], db[1], 1u);
                umma_f16(tmem + 3 * SP_TN, da[3], db[0], 1u);
                umma_f16(tmem + 3 * SP_TN, da[0], db[4], 1u);
                umma_f16(tmem + 3 * SP_TN, da[1], db[3], 1u);
                umma_f16(tmem + 3 * SP_TN, da[2], db[2], 1u);
                umma_f16(tmem + 3 * SP_TN, da[3], db[1], 1u);
                umma_f16(tmem + 3 * SP_TN, da[4], db[0], 1u);
                umma_commit(&bar_empty[s]);
            }
            umma_commit(&bar_done);   // arrives once every MMA issued above has completed
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32w..32w+31 = tile rows
        const bool ok = mbar_wait(&bar_done, 0, a.err, a.wait_ns);
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (ok) {
            const int r = warp * 32 + lane;
            const int64_t i = (int64_t)rb * SP_TM + r;
            const bool row_ok = i < a.M;
            const int e = row_ok ? a.eexp[(int64_t)z * a.M + i] : 0;
            for (int c0 = 0; c0 < SP_TN; c0 += 32) {
                uint32_t g0[32], g1[32], g2[32], g3[32];
                const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + c0;
                SP_LD32(base + 0 * SP_TN, g0);
                SP_LD32(base + 1 * SP_TN, g1);
                SP_LD32(base + 2 * SP_TN, g2);
                SP_LD32(base + 3 * SP_TN, g3);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (!row_ok) continue;
#pragma unroll
                for (int q = 0; q < 32; q += 2) {
                    const int jr = nb * SP_TN + c0 + q;   // real column (even: Re)
                    const int j = jr >> 1;
                    if (j >= a.N) break;
                    // weight-2 and -3 groups are exact and their sum is kept exact as an FP32 pair
                    // (s, t); the weight >= 4 groups are 2^-14 of them and join t, rounding at ~2^-38
                    // of the result.  Two conversions and one FP64 add per value (the FP64 pipe is
                    // the epilogue's limit); the power-of-two scale goes into the exponent field.
                    const int sc = e + a.fexp[j] - 2 * SPLIT_BITS;   // each operand carries 2^-7
                    const double re = scale_pow2(recombine(g0[q], g1[q], g2[q], g3[q]), sc);
                    const double im = scale_pow2(recombine(g0[q + 1], g1[q + 1], g2[q + 1], g3[q + 1]), sc);
                    cplx v = mk(re, im);
                    cplx *dst = a.C + (int64_t)z * a.c_sb + i * a.c_si + (int64_t)j * a.c_sj;
                    if (a.accumulate) v = cadd(v, *dst);
                    *dst = v;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // After a wait gave up, copies may still be in flight and MMAs still running: the last
    // round of each stage lands and every issued MMA completes before the CTA frees its TMEM
    // and leaves (waits bounded by SP_WAIT_NS; without an error they return at once).
    if (warp == 4 && lane == 0)
        for (int ks = issued - 1; ks >= 0 && ks >= issued - SP_STAGES; ks--)
            mbar_drain(&bar_full[ks % SP_STAGES], (uint32_t)((ks / SP_STAGES) & 1));
    if (warp == 5 && lane == 0) mbar_drain(&bar_done, 0);
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(4 * SP_TN));
    }
}

// Persistent form of the same product.  Work items are 128 x 64 output tiles (half of a
// 128-column B tile); each CTA takes items grid-stride.  Two accumulator sets of four groups
// x 64 columns fill the 512 TMEM columns, so the MMAs of one item run while the epilogue
// warps recombine the previous one: the epilogue, bound by the FP64 pipe, overlaps the
// tensor work instead of following it.  Roles and stage pipeline as in sp_gemm_kernel, with
// the stage and item counters running across items.
constexpr int SPP_STAGES = 5;
constexpr int SPP_STAGE_BYTES = SPLIT_S * SP_TILE_BYTES + SPLIT_S * (SP_TILE_BYTES / 2);   // 30 KB
constexpr int SPP_SMEM = SPP_STAGES * SPP_STAGE_BYTES + 1024;

__global__ void __launch_bounds__(SP_THREADS, 1) sp_gemm_persist_kernel(SplitArgs a) {
    extern __shared__ __align__(1024) unsigned char sp_raw[];
    __shared__ __align__(8) uint64_t bar_full[SPP_STAGES], bar_empty[SPP_STAGES], acc_full[2], acc_empty[2], bar_drain;
    __shared__ uint32_t s_tmem;
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(sp_raw) + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nnh = (2 * a.N + SPP_TN - 1) / SPP_TN;        // 64-column halves holding output columns
    const int64_t items = (int64_t)a.nz * a.nrb * nnh;
    const int nks = a.nks;
    auto item_coords = [&](int64_t t, int &z, int &rb, int &nh) {
        z = (int)(t / ((int64_t)a.nrb * nnh));
        const int64_t r = t % ((int64_t)a.nrb * nnh);
        if (a.order) {
            rb = (int)(r % a.nrb);
            nh = (int)(r / a.nrb);
        } else {
            rb = (int)(r / nnh);
            nh = (int)(r % nnh);
        }
    };

    if (threadIdx.x == 0) {
        for (int q = 0; q < SPP_STAGES; q++) {
            mbar_init(&bar_full[q], 1);
            mbar_init(&bar_empty[q], 1);
        }
        for (int q = 0; q < 2; q++) {
            mbar_init(&acc_full[q], 1);
            mbar_init(&acc_empty[q], 4);   // one arrival per epilogue warp
        }
        mbar_init(&bar_drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {   // 2 sets x 4 groups x 64 columns = 512 TMEM columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;

    int64_t issued = 0;   // producer: stage rounds whose copies were issued
    if (warp == 4) {
        if (lane == 0) {   // producer
            int64_t it = 0;
            bool ok = true;
            for (int64_t t = blockIdx.x; t < items && ok; t += gridDim.x) {
                int z, rb, nh;
                item_coords(t, z, rb, nh);
                const int nb = nh >> 1, half = nh & 1;
                for (int ks = 0; ks < nks; ks++, it++) {
                    const int s = (int)(it % SPP_STAGES);
                    if (it >= SPP_STAGES && !mbar_wait(&bar_empty[s], (uint32_t)(((it / SPP_STAGES) - 1) & 1), a.err, a.wait_ns)) {
                        ok = false;
                        break;
                    }
                    unsigned char *st = smem + s * SPP_STAGE_BYTES;
                    mbar_expect_tx(&bar_full[s], SPP_STAGE_BYTES);
                    for (int p = 0; p < SPLIT_S; p++) {
                        const int64_t ta = (((int64_t)p * a.nz + z) * a.nrb + rb) * nks + ks;
                        bulk_g2s(st + p * SP_TILE_BYTES, reinterpret_cast<const char *>(a.As) + ta * SP_TILE_BYTES,
                                 SP_TILE_BYTES, &bar_full[s]);
                        const int64_t tb = ((int64_t)p * a.nnb + nb) * nks + ks;
                        bulk_g2s(st + SPLIT_S * SP_TILE_BYTES + p * (SP_TILE_BYTES / 2),
                                 reinterpret_cast<const char *>(a.Bs) + tb * SP_TILE_BYTES + half * (SP_TILE_BYTES / 2),
                                 SP_TILE_BYTES / 2, &bar_full[s]);
                    }
                }
            }
            issued = it;
        }
    } else if (warp == 5) {
        if (lane == 0) {   // MMA issuer
            int64_t it = 0, tl = 0;
            bool ok = true;
            for (int64_t t = blockIdx.x; t < items && ok; t += gridDim.x, tl++) {
                const int b = (int)(tl & 1);
                if (tl >= 2 && !mbar_wait(&acc_empty[b], (uint32_t)(((tl >> 1) - 1) & 1), a.err, a.wait_ns)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t acc = tmem + (uint32_t)(b * 4 * SPP_TN);
                for (int ks = 0; ks < nks; ks++, it++) {
                    const int s = (int)(it % SPP_STAGES);
                    if (!mbar_wait(&bar_full[s], (uint32_t)((it / SPP_STAGES) & 1), a.err, a.wait_ns)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const unsigned char *st = smem + s * SPP_STAGE_BYTES;
                    uint64_t da[SPLIT_S], db[SPLIT_S];
#pragma unroll
                    for (int p = 0; p < SPLIT_S; p++) {
                        da[p] = sp_desc(st + p * SP_TILE_BYTES, a.lbo, a.sbo);
                        db[p] = sp_desc(st + SPLIT_S * SP_TILE_BYTES + p * (SP_TILE_BYTES / 2), a.lbo, a.sbo);
                    }
                    const uint32_t first = ks > 0 ? 1u : 0u;
                    umma_f16_n64(acc + 0 * SPP_TN, da[0], db[0], first);
                    umma_f16_n64(acc + 1 * SPP_TN, da[0], db[1], first);
                    umma_f16_n64(acc + 1 * SPP_TN, da[1], db[0], 1u);
                    umma_f16_n64(acc + 2 * SPP_TN, da[0], db[2], first);
                    umma_f16_n64(acc + 2 * SPP_TN, da[1], db[1], 1u);
                    umma_f16_n64(acc + 2 * SPP_TN, da[2], db[0], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[0], db[3], first);
                    umma_f16_n64(acc + 3 * SPP_TN, da[1], db[2], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[2], db[1], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[3], db[0], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[0], db[4], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[1], db[3], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[2], db[2], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[3], db[1], 1u);
                    umma_f16_n64(acc + 3 * SPP_TN, da[4], db[0], 1u);
                    umma_commit(&bar_empty[s]);
                }
                if (ok) umma_commit(&acc_full[b]);
            }
            umma_commit(&bar_drain);   // arrives once every MMA issued above has completed
            mbar_drain(&bar_drain, 0);
        }
    } else {
        // epilogue warps 0-3: warp w owns TMEM lanes 32w..32w+31 = tile rows
        int64_t tl = 0;
        for (int64_t t = blockIdx.x; t < items; t += gridDim.x, tl++) {
            const int b = (int)(tl & 1);
            if (!mbar_wait(&acc_full[b], (uint32_t)((tl >> 1) & 1), a.err, a.wait_ns)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            int z, rb, nh;
            item_coords(t, z, rb, nh);
            const int r = warp * 32 + lane;
            const int64_t i = (int64_t)rb * SP_TM + r;
            const bool row_ok = i < a.M;
            const int e = row_ok ? a.eexp[(int64_t)z * a.M + i] : 0;
            const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * 4 * SPP_TN);
            for (int c0 = 0; c0 < SPP_TN; c0 += 32) {
                uint32_t g0[32], g1[32], g2[32], g3[32];
                SP_LD32(base + 0 * SPP_TN + c0, g0);
                SP_LD32(base + 1 * SPP_TN + c0, g1);
                SP_LD32(base + 2 * SPP_TN + c0, g2);
                SP_LD32(base + 3 * SPP_TN + c0, g3);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (c0 + 32 >= SPP_TN) {   // the accumulator set is read: hand it back to the MMAs
                    asm volatile("tcgen05.fence::before_thread_sync;");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&acc_empty[b]);
                }
                if (!row_ok) continue;
#pragma unroll
                for (int q = 0; q < 32; q += 2) {
                    const int jr = nh * SPP_TN + c0 + q;   // real column (even: Re)
                    const int j = jr >> 1;
                    if (j >= a.N) break;
                    const int sc = e + a.fexp[j] - 2 * SPLIT_BITS;
                    const double re = scale_pow2(recombine(g0[q], g1[q], g2[q], g3[q]), sc);
                    const double im = scale_pow2(recombine(g0[q + 1], g1[q + 1], g2[q + 1], g3[q + 1]), sc);
                    cplx v = mk(re, im);
                    cplx *dst = a.C + (int64_t)z * a.c_sb + i * a.c_si + (int64_t)j * a.c_sj;
                    if (a.accumulate) v = cadd(v, *dst);
                    *dst = v;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // copies still in flight after any role gave up land before the CTA leaves (the MMA issuer
    // has already waited for its MMAs through bar_drain); without an error this returns at once
    if (warp == 4 && lane == 0)
        for (int64_t j = issued - 1; j >= 0 && j >= issued - SPP_STAGES; j--)
            mbar_drain(&bar_full[j % SPP_STAGES], (uint32_t)((j / SPP_STAGES) & 1));
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

// ------------------------------------------------------------------------- accurate form
// The same product with SPA_S = 7 slices per operand (49 bits), for the contractions whose
// errors the metric's inverse amplifies (the Gram metric K = G G^H, G v and P^H (G v) of the A
// and C blocks): the products with p + q <= 6 (28 of 49) go to five TMEM accumulators of 64
// columns by weight p + q = 0, 1, 2, 3 and >= 4.  The first three are exact (integer partial
// sums below 2^24 for K' <= 1024 real); the weight-3 group holds terms 2^-21 of the leading one
// and the last 2^-28, so their FP32 rounding is ~2^-45 of the result, the same size as the
// omitted products (weights >= 7, 2^-49 each).  The epilogue converts the five groups to FP64
// and adds them smallest first.  Result: ~2^-45 of max|row of A| * max|column of B| per term.
// One 128 x 64 output tile per CTA; producer, MMA issuer and epilogue warps as sp_gemm_kernel.
constexpr int SPA_S = 7;
constexpr int SPA_TN = 64;
constexpr int SPA_GROUPS = 5;
constexpr int SPA_STAGES = 4;
constexpr int SPA_STAGE_BYTES = SPA_S * SP_TILE_BYTES + SPA_S * (SP_TILE_BYTES / 2);   // 42 KB
constexpr int SPA_SMEM = SPA_STAGES * SPA_STAGE_BYTES + 1024;

__global__ void __launch_bounds__(SP_THREADS, 1) sp_gemm_acc_kernel(SplitArgs a) {
    extern __shared__ __align__(1024) unsigned char sp_raw[];
    __shared__ __align__(8) uint64_t bar_full[SPA_STAGES], bar_empty[SPA_STAGES], bar_done;
    __shared__ uint32_t s_tmem;
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(sp_raw) + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nnh = (2 * a.N + SPA_TN - 1) / SPA_TN;        // 64-column halves of the 128-column B tiles
    const int rb = (int)(blockIdx.x / (unsigned)nnh);
    const int nh = (int)(blockIdx.x % (unsigned)nnh);
    const int nb = nh >> 1, half = nh & 1;
    const int z = blockIdx.z;

    if (threadIdx.x == 0) {
        for (int q = 0; q < SPA_STAGES; q++) {
            mbar_init(&bar_full[q], 1);
            mbar_init(&bar_empty[q], 1);
        }
        mbar_init(&bar_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {   // 5 groups x 64 columns used of a 512-column allocation (a power of two)
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;
    const int nks = a.nks;
    int issued = 0;

    if (warp == 4) {
        if (lane == 0) {   // producer: SPA_S A tiles (4 KB) and SPA_S B half-tiles (2 KB) per stage
            for (int ks = 0; ks < nks; ks++) {
                const int st_i = ks % SPA_STAGES;
                if (ks >= SPA_STAGES &&
                    !mbar_wait(&bar_empty[st_i], ((ks / SPA_STAGES) - 1) & 1, a.err, a.wait_ns))
                    break;
                issued = ks + 1;
                unsigned char *st = smem + st_i * SPA_STAGE_BYTES;
                mbar_expect_tx(&bar_full[st_i], SPA_STAGE_BYTES);
                for (int p = 0; p < SPA_S; p++) {
                    const int64_t ta = (((int64_t)p * a.nz + z) * a.nrb + rb) * nks + ks;
                    bulk_g2s(st + p * SP_TILE_BYTES, reinterpret_cast<const char *>(a.As) + ta * SP_TILE_BYTES,
                             SP_TILE_BYTES, &bar_full[st_i]);
                    const int64_t tb = ((int64_t)p * a.nnb + nb) * nks + ks;
                    bulk_g2s(st + SPA_S * SP_TILE_BYTES + p * (SP_TILE_BYTES / 2),
                             reinterpret_cast<const char *>(a.Bs) + tb * SP_TILE_BYTES + half * (SP_TILE_BYTES / 2),
                             SP_TILE_BYTES / 2, &bar_full[st_i]);
                }
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {   // MMA issuer: 28 products per K step, by weight p + q
            for (int ks = 0; ks < nks; ks++) {
                const int st_i = ks % SPA_STAGES;
                if (!mbar_wait(&bar_full[st_i], (ks / SPA_STAGES) & 1, a.err, a.wait_ns)) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const unsigned char *st = smem + st_i * SPA_STAGE_BYTES;
                uint64_t da[SPA_S], db[SPA_S];
#pragma unroll
                for (int p = 0; p < SPA_S; p++) {
                    da[p] = sp_desc(st + p * SP_TILE_BYTES, a.lbo, a.sbo);
                    db[p] = sp_desc(st + SPA_S * SP_TILE_BYTES + p * (SP_TILE_BYTES / 2), a.lbo, a.sbo);
                }
#pragma unroll
                for (int w = 0; w < SPA_S; w++) {
                    const int g = w < SPA_GROUPS - 1 ? w : SPA_GROUPS - 1;
#pragma unroll
                    for (int p = 0; p <= w; p++) {
                        // the first product into a group at the first K step overwrites it
                        const bool first = ks == 0 && p == 0 && w < SPA_GROUPS;
                        umma_f16_n64(tmem + (uint32_t)(g * SPA_TN), da[p], db[w - p], first ? 0u : 1u);
                    }
                }
                umma_commit(&bar_empty[st_i]);
            }
            umma_commit(&bar_done);   // arrives once every MMA issued above has completed
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32w..32w+31 = tile rows
        const bool ok = mbar_wait(&bar_done, 0, a.err, a.wait_ns);
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (ok) {
            const int r = warp * 32 + lane;
            const int64_t i = (int64_t)rb * SP_TM + r;
            const bool row_ok = i < a.M;
            const int e = row_ok ? a.eexp[(int64_t)z * a.M + i] : 0;
            for (int c0 = 0; c0 < SPA_TN; c0 += 32) {
                uint32_t g0[32], g1[32], g2[32], g3[32], g4[32];
                const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + c0;
                SP_LD32(base + 0 * SPA_TN, g0);
                SP_LD32(base + 1 * SPA_TN, g1);
                SP_LD32(base + 2 * SPA_TN, g2);
                SP_LD32(base + 3 * SPA_TN, g3);
                SP_LD32(base + 4 * SPA_TN, g4);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (!row_ok) continue;
#pragma unroll
                for (int q = 0; q < 32; q += 2) {
                    const int jr = nh * SPA_TN + c0 + q;   // real column (even: Re)
                    const int j = jr >> 1;
                    if (j >= a.N) break;
                    const int sc = e + a.fexp[j] - 2 * SPLIT_BITS;
                    double v2[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        double v = (double)__uint_as_float(g4[q + h]);
                        v += (double)__uint_as_float(g3[q + h]);
                        v += (double)__uint_as_float(g2[q + h]);
                        v += (double)__uint_as_float(g1[q + h]);
                        v += (double)__uint_as_float(g0[q + h]);
                        v2[h] = scale_pow2(v, sc);
                    }
                    cplx val = mk(v2[0], v2[1]);
                    cplx *dst = a.C + (int64_t)z * a.c_sb + i * a.c_si + (int64_t)j * a.c_sj;
                    if (a.accumulate) val = cadd(val, *dst);
                    *dst = val;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // after a wait gave up: copies in flight land and issued MMAs complete before TMEM is freed
    if (warp == 4 && lane == 0)
        for (int ks = issued - 1; ks >= 0 && ks >= issued - SPA_STAGES; ks--)
            mbar_drain(&bar_full[ks % SPA_STAGES], (uint32_t)((ks / SPA_STAGES) & 1));
    if (warp == 5 && lane == 0) mbar_drain(&bar_done, 0);
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

// ------------------------------------------------------------------------- host driver
// C = A * op(B) (+ C when accumulate), complex FP64 in and out, through the split path.
// Large operand: element (i, k) of batch z at A[z*a_sb + i*a_si + k*a_sk], i < M, k < K.
// Small operand: op(B)(k, j) = B[k + j ldb], or B[j + k ldb] when opb & 2; conjugated when
// opb & 1; j < N.
// Output: C[z*c_sb + i*c_si + j*c_sj].
void zgemm_split(Context &c, int M, int N, int K, int batch, const cplx *A, int64_t a_si, int64_t a_sk, int64_t a_sb,
                 const cplx *B, int64_t ldb, int opb, cplx *C, int64_t c_si, int64_t c_sj, int64_t c_sb,
                 bool accumulate, int lbo, int sbo) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (batch > 65535) {   // grid z limit: chain batch chunks
        for (int z0 = 0; z0 < batch; z0 += 65535)
            zgemm_split(c, M, N, K, std::min(65535, batch - z0), A + z0 * a_sb, a_si, a_sk, a_sb, B, ldb, opb,
                        C + z0 * c_sb, c_si, c_sj, c_sb, accumulate, lbo, sbo);
        return;
    }
    const int kmax = SP_KMAX / 2;   // complex K per launch
    if (K > kmax) {   // exact FP32 groups need K' <= SP_KMAX: chain K chunks through C
        for (int k0 = 0; k0 < K; k0 += kmax) {
            const int kc = std::min(kmax, K - k0);
            zgemm_split(c, M, N, kc, batch, A + k0 * a_sk, a_si, a_sk, a_sb, (opb & 2) ? B + k0 * ldb : B + k0, ldb, opb,
                        C, c_si, c_sj, c_sb,
                        accumulate || k0 > 0, lbo, sbo);
        }
        return;
    }
    GemmTrace trace(c, "split", M, N, K, batch);
    const int nks = (2 * K + SP_TK - 1) / SP_TK;
    const int nrb = (M + SP_TM - 1) / SP_TM;
    const int nnb = (2 * N + SP_TN - 1) / SP_TN;
    const size_t tiles_a = (size_t)SPLIT_S * batch * nrb * nks, tiles_b = (size_t)SPLIT_S * nnb * nks;
    __nv_bfloat16 *As = wsget<__nv_bfloat16>(c, "split.A", tiles_a * SP_TILE_BYTES / 2);
    __nv_bfloat16 *Bs = wsget<__nv_bfloat16>(c, "split.B", tiles_b * SP_TILE_BYTES / 2);
    int *eexp = wsget<int>(c, "split.e", (size_t)M * batch);
    int *fexp = wsget<int>(c, "split.f", (size_t)N);
    int *err = wsget<int>(c, "split.err", 1);
    // B' tiles may have padding columns beyond 2N: zero them all first.  The error flag is
    // reset by split_reset() at the start of a solve and read by split_error() at its end.
    DCG_CUDA(cudaMemsetAsync(Bs, 0, tiles_b * SP_TILE_BYTES, c.stream));
    launch_rowexp(c, M, K, batch, A, a_si, a_sk, a_sb, eexp);
    {
        const int64_t work = (int64_t)nrb * SP_TM * nks * (SP_TK / 8);
        dim3 g(grid1d(work, 256), batch);
        sp_slice_a_kernel<SPLIT_S><<<g, 256, 0, c.stream>>>(M, K, A, a_si, a_sk, a_sb, eexp, batch, nrb, nks, As);
        DCG_LAUNCHED(c);
    }
    sp_slice_b_kernel<SPLIT_S><<<N, 128, 0, c.stream>>>(K, N, B, ldb, opb, nnb, nks, Bs, fexp);
    DCG_LAUNCHED(c);
    DCG_CUDA(cudaFuncSetAttribute(sp_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SP_SMEM));
    SplitArgs sa;
    sa.As = As;
    sa.Bs = Bs;
    sa.eexp = eexp;
    sa.fexp = fexp;
    sa.C = C;
    sa.c_si = c_si;
    sa.c_sj = c_sj;
    sa.c_sb = c_sb;
    sa.M = M;
    sa.N = N;
    sa.nz = batch;
    sa.nrb = nrb;
    sa.nnb = nnb;
    sa.nks = nks;
    sa.lbo = lbo;
    sa.sbo = sbo;
    sa.accumulate = accumulate ? 1 : 0;
    sa.order = 0;
    sa.err = err;
    sa.wait_ns = c.wait_limit_ns ? c.wait_limit_ns : SP_WAIT_NS;
    dim3 grid((unsigned)((int64_t)nrb * nnb), 1, batch);
    // CTA raster tuned per shape when both orders have more than one block to order; trial
    // launches overwrite C, so only non-accumulating products are timed
    const double tensor_work = 15.0 * 8.0 * (double)M * N * K * batch;
    // kernel and CTA raster, tuned per shape: candidate q = raster (q & 1), persistent (q & 2);
    // products under ~0.1 ms of tensor work keep candidate 0
    DCG_CUDA(cudaFuncSetAttribute(sp_gemm_persist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SPP_SMEM));
    const int64_t pitems = (int64_t)batch * nrb * ((2 * N + SPP_TN - 1) / SPP_TN);
    const unsigned pgrid = (unsigned)std::min<int64_t>(pitems, std::max(1, c.num_sms));
    auto launch = [&](int q) {
        SplitArgs t = sa;
        t.order = q & 1;
        if (q & 2) sp_gemm_persist_kernel<<<pgrid, SP_THREADS, SPP_SMEM, c.stream>>>(t);
        else sp_gemm_kernel<<<grid, SP_THREADS, SP_SMEM, c.stream>>>(t);
        DCG_LAUNCHED(c);
    };
    const TuneKey key{TUNE_SPLIT_KERNEL, batch, M, N, K, 0};
    int pick;
    const char *force = getenv("DCG_SPLIT_KERNEL");   // diagnostic: a fixed candidate 0-3
    if (force && force[0] >= '0' && force[0] <= '3' && force[1] == 0) pick = force[0] - '0';
    else pick = autotune(c, key, 4, !accumulate && tensor_work >= 1.0e11, launch);
    {
        // tensor work: 15 slice products, each a real GEMM of M x 2N x 2K
        FamScope fs(c, DCG_FAM_SPLIT_MMA, tensor_work);
        launch(pick);
    }
}

// C = A * op(B) (+ C) as zgemm_split, through the accurate seven-slice kernel (~2^-45 of
// max|row of A| * max|column of B| per term instead of ~2^-36).  No tuning: one kernel.
void zgemm_split_acc(Context &c, int M, int N, int K, int batch, const cplx *A, int64_t a_si, int64_t a_sk,
                     int64_t a_sb, const cplx *B, int64_t ldb, int opb, cplx *C, int64_t c_si, int64_t c_sj,
                     int64_t c_sb, bool accumulate) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (batch > 65535) {
        for (int z0 = 0; z0 < batch; z0 += 65535)
            zgemm_split_acc(c, M, N, K, std::min(65535, batch - z0), A + z0 * a_sb, a_si, a_sk, a_sb, B, ldb, opb,
                            C + z0 * c_sb, c_si, c_sj, c_sb, accumulate);
        return;
    }
    const int kmax = SP_KMAX / 2;
    if (K > kmax) {   // exact FP32 groups need K' <= SP_KMAX: chain K chunks through C
        for (int k0 = 0; k0 < K; k0 += kmax) {
            const int kc = std::min(kmax, K - k0);
            zgemm_split_acc(c, M, N, kc, batch, A + k0 * a_sk, a_si, a_sk, a_sb, (opb & 2) ? B + k0 * ldb : B + k0,
                            ldb, opb, C, c_si, c_sj, c_sb, accumulate || k0 > 0);
        }
        return;
    }
    if (K <= 0) {   // empty sum
        if (!accumulate) {
            const cplx zero = mk(0.0, 0.0);
            zgemm(c, OP_N, OP_N, M, N, 0, zero, A, std::max<int64_t>(a_sk, 1), 0, B, std::max<int64_t>(ldb, 1), 0, zero,
                  C, c_sj, c_sb, batch);
        }
        return;
    }
    GemmTrace trace(c, "split_acc", M, N, K, batch);
    const int nks = (2 * K + SP_TK - 1) / SP_TK;
    const int nrb = (M + SP_TM - 1) / SP_TM;
    const int nnb = (2 * N + SP_TN - 1) / SP_TN;
    const int nnh = (2 * N + SPA_TN - 1) / SPA_TN;
    const size_t tiles_a = (size_t)SPA_S * batch * nrb * nks, tiles_b = (size_t)SPA_S * nnb * nks;
    __nv_bfloat16 *As = wsget<__nv_bfloat16>(c, "splitacc.A", tiles_a * SP_TILE_BYTES / 2);
    __nv_bfloat16 *Bs = wsget<__nv_bfloat16>(c, "splitacc.B", tiles_b * SP_TILE_BYTES / 2);
    int *eexp = wsget<int>(c, "splitacc.e", (size_t)M * batch);
    int *fexp = wsget<int>(c, "splitacc.f", (size_t)N);
    int *err = wsget<int>(c, "split.err", 1);
    DCG_CUDA(cudaMemsetAsync(Bs, 0, tiles_b * SP_TILE_BYTES, c.stream));
    launch_rowexp(c, M, K, batch, A, a_si, a_sk, a_sb, eexp);
    {
        const int64_t work = (int64_t)nrb * SP_TM * nks * (SP_TK / 8);
        dim3 g(grid1d(work, 256), batch);
        sp_slice_a_kernel<SPA_S><<<g, 256, 0, c.stream>>>(M, K, A, a_si, a_sk, a_sb, eexp, batch, nrb, nks, As);
        DCG_LAUNCHED(c);
    }
    sp_slice_b_kernel<SPA_S><<<N, 128, 0, c.stream>>>(K, N, B, ldb, opb, nnb, nks, Bs, fexp);
    DCG_LAUNCHED(c);
    DCG_CUDA(cudaFuncSetAttribute(sp_gemm_acc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SPA_SMEM));
    SplitArgs sa;
    sa.As = As;
    sa.Bs = Bs;
    sa.eexp = eexp;
    sa.fexp = fexp;
    sa.C = C;
    sa.c_si = c_si;
    sa.c_sj = c_sj;
    sa.c_sb = c_sb;
    sa.M = M;
    sa.N = N;
    sa.nz = batch;
    sa.nrb = nrb;
    sa.nnb = nnb;
    sa.nks = nks;
    sa.lbo = c.split_lbo;
    sa.sbo = c.split_sbo;
    sa.accumulate = accumulate ? 1 : 0;
    sa.order = 0;
    sa.err = err;
    sa.wait_ns = c.wait_limit_ns ? c.wait_limit_ns : SP_WAIT_NS;
    const double tensor_work = 28.0 * 8.0 * (double)M * N * K * batch;   // 28 slice products
    FamScope fs(c, DCG_FAM_SPLIT_MMA, tensor_work);
    sp_gemm_acc_kernel<<<dim3((unsigned)((int64_t)nrb * nnh), 1, batch), SP_THREADS, SPA_SMEM, c.stream>>>(sa);
    DCG_LAUNCHED(c);
}

void split_reset(Context &c) {
    int *err = wsget<int>(c, "split.err", 1);
    DCG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
}

// 0 when no split GEMM wait ran out since split_reset(), else 1 (synchronises the stream)
int split_error(Context &c) {
    int *err = wsget<int>(c, "split.err", 1);
    int h = 0;
    DCG_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    return h;
}

}  // namespace dcg
