// Dense FP64 complex linear algebra on the device: workspace, GEMM, Hermitian fill,
// deterministic sums and the LU solve (Golub & Van Loan, Matrix Computations, 4th ed.,
// 3.4: partial pivoting).  The Hermitian eigensolver lives in dcg_eig.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "dcg_common.cuh"

namespace dcg {

// ===================================================================== workspace
void *Workspace::get(const std::string &name, size_t bytes) {
    Buf &b = bufs_[name];
    if (b.bytes >= bytes && b.p) return b.p;
    if (b.p) {
        cudaFree(b.p);
        total_ -= b.bytes;
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t alloc = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&b.p, alloc);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        throw Error{DCG_E_NOMEM, "device allocation of " + std::to_string(alloc) + " bytes for " + name +
                                     " failed: " + cudaGetErrorString(e)};
    }
    b.bytes = alloc;
    total_ += alloc;
    return b.p;
}

void *Workspace::host(const std::string &name, size_t bytes) {
    Buf &b = host_[name];
    if (b.bytes >= bytes && b.p) return b.p;
    if (b.p) {
        cudaFreeHost(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    const size_t alloc = bytes < 256 ? 256 : bytes;
    const cudaError_t e = cudaHostAlloc(&b.p, alloc, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        throw Error{DCG_E_NOMEM, "page-locked allocation for " + name + " failed: " + cudaGetErrorString(e)};
    }
    b.bytes = alloc;
    return b.p;
}

void Workspace::release_all() {
    for (auto &kv : bufs_)
        if (kv.second.p) cudaFree(kv.second.p);
    bufs_.clear();
    for (auto &kv : host_)
        if (kv.second.p) cudaFreeHost(kv.second.p);
    host_.clear();
    total_ = 0;
}

// ===================================================================== block reductions
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum (fixed reduction tree); result valid in every thread.
__device__ double block_sum(double v, double *sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    double r = sh[0];
    __syncthreads();
    return r;
}

// ===================================================================== ZGEMM
// 256 threads as TYN x (256 / TYN), each owning a 4 x 4 block of outputs spaced TYN rows and
// 256/TYN columns apart: tiles of 64 x 64 (TYN 16), 32 x 128 (TYN 8) or 128 x 32 (TYN 32).
// A GB300 SM retires about two FP64 FMAs per clock, so the useful fraction of a tile is the
// fraction of the GPU's FP64 rate a skinny product gets: the autotuner picks the tile.
constexpr int kZgTiles = 3;
constexpr int kZgTyn[kZgTiles] = {16, 8, 32};

template <int OPA, int OPB, int TYN>
__global__ void __launch_bounds__(256) zgemm_kernel(int m, int n, int k, cplx alpha, const cplx *__restrict__ A,
                                                    int64_t lda, int64_t sa, const cplx *__restrict__ B,
                                                    int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc,
                                                    int64_t sc, int zoff, int upper) {
    constexpr int TXN = 256 / TYN, BM = 4 * TYN, BN = 4 * TXN, BK = 16;
    __shared__ cplx As[BK][BM + 1];
    __shared__ cplx Bs[BK][BN + 1];
    const int64_t bz = (int64_t)blockIdx.z + zoff;
    A += bz * sa;
    B += bz * sb;
    C += bz * sc;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (upper && m0 >= n0 + BN) return;   // tile strictly below the diagonal (Hermitian product, upper half)
    const int tx = threadIdx.x % TXN, ty = threadIdx.x / TXN;
    cplx acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = mk(0.0, 0.0);
    for (int k0 = 0; k0 < k; k0 += BK) {
        for (int e = threadIdx.x; e < BM * BK; e += 256) {
            int i, kk;
            if (OPA == OP_N || OPA == OP_R) {
                i = e % BM;
                kk = e / BM;
            } else {
                kk = e % BK;
                i = e / BK;
            }
            int gi = m0 + i, gk = k0 + kk;
            cplx v = mk(0.0, 0.0);
            if (gi < m && gk < k) {
                v = (OPA == OP_N || OPA == OP_R) ? A[gi + (int64_t)gk * lda] : A[gk + (int64_t)gi * lda];
                if (OPA == OP_C || OPA == OP_R) v = cconj(v);
            }
            As[kk][i] = v;
        }
        for (int e = threadIdx.x; e < BN * BK; e += 256) {
            int j, kk;
            if (OPB == OP_N || OPB == OP_R) {
                kk = e % BK;
                j = e / BK;
            } else {
                j = e % BN;
                kk = e / BN;
            }
            int gj = n0 + j, gk = k0 + kk;
            cplx v = mk(0.0, 0.0);
            if (gj < n && gk < k) {
                v = (OPB == OP_N || OPB == OP_R) ? B[gk + (int64_t)gj * ldb] : B[gj + (int64_t)gk * ldb];
                if (OPB == OP_C || OPB == OP_R) v = cconj(v);
            }
            Bs[kk][j] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < BK; kk++) {
            cplx a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                a[q] = As[kk][ty + TYN * q];
                b[q] = Bs[kk][tx + TXN * q];
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) cfma(acc[p][q], a[p], b[q]);
        }
        __syncthreads();
    }
    const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
#pragma unroll
    for (int p = 0; p < 4; p++) {
        int gi = m0 + ty + TYN * p;
        if (gi >= m) continue;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int gj = n0 + tx + TXN * q;
            if (gj >= n) continue;
            cplx r = cmul(alpha, acc[p][q]);
            int64_t o = gi + (int64_t)gj * ldc;
            if (use_beta) r = cadd(r, cmul(beta, C[o]));
            C[o] = r;
        }
    }
}

// ---- small-dimension GEMMs of the 4-index transformation.  When the contracted index
// and the small output index are at most SMALL_D (an active or inactive orbital dimension),
// the GEMM is memory-bound: the small matrix is staged in shared memory and the large
// operand is streamed once.  Each thread owns one row (right-small) or one column
// (left-small) and SMALL_G consecutive outputs of it.
constexpr int SMALL_D = 32, SMALL_G = 8;

// C(m x n) = alpha * A(m x k) * op(B)(k x n) + beta * C, op(B) = B or conj(B); k, n <= SMALL_D.
template <int OPB>
__global__ void __launch_bounds__(256) zgemm_rsmall_kernel(int m, int n, int k, cplx alpha, const cplx *__restrict__ A,
                                                           int64_t lda, int64_t sa, const cplx *__restrict__ B,
                                                           int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc,
                                                           int64_t sc, int z0) {
    __shared__ cplx Bs[SMALL_D][SMALL_D];
    const int z = z0 + blockIdx.z;
    A += (int64_t)z * sa;
    B += (int64_t)z * sb;
    C += (int64_t)z * sc;
    for (int x = threadIdx.x + blockDim.x * threadIdx.y; x < k * n; x += blockDim.x * blockDim.y) {
        const int kk = x % k, j = x / k;
        cplx v = B[kk + (int64_t)j * ldb];
        if (OPB == OP_R) v = cconj(v);
        Bs[kk][j] = v;
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j0 = threadIdx.y * SMALL_G;
    if (i >= m || j0 >= n) return;
    cplx acc[SMALL_G];
#pragma unroll
    for (int q = 0; q < SMALL_G; q++) acc[q] = mk(0.0, 0.0);
    for (int kk = 0; kk < k; kk++) {
        const cplx a = A[i + (int64_t)kk * lda];
#pragma unroll
        for (int q = 0; q < SMALL_G; q++)
            if (j0 + q < n) cfma(acc[q], a, Bs[kk][j0 + q]);
    }
    const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
#pragma unroll
    for (int q = 0; q < SMALL_G; q++) {
        if (j0 + q >= n) break;
        const int64_t o = i + (int64_t)(j0 + q) * ldc;
        cplx r = cmul(alpha, acc[q]);
        if (use_beta) r = cadd(r, cmul(beta, C[o]));
        C[o] = r;
    }
}

// C(m x n) = alpha * A^H(m x k) * B(k x n) + beta * C with A (k x m); m, k <= SMALL_D.
__global__ void __launch_bounds__(256) zgemm_lsmall_kernel(int m, int n, int k, cplx alpha, const cplx *__restrict__ A,
                                                           int64_t lda, int64_t sa, const cplx *__restrict__ B,
                                                           int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc,
                                                           int64_t sc, int z0) {
    __shared__ cplx As[SMALL_D][SMALL_D];   // As[kk][i] = conj(A(kk, i))
    const int z = z0 + blockIdx.z;
    A += (int64_t)z * sa;
    B += (int64_t)z * sb;
    C += (int64_t)z * sc;
    for (int x = threadIdx.x + blockDim.x * threadIdx.y; x < k * m; x += blockDim.x * blockDim.y) {
        const int kk = x % k, i = x / k;
        As[kk][i] = cconj(A[kk + (int64_t)i * lda]);
    }
    __syncthreads();
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int i0 = threadIdx.y * SMALL_G;
    if (j >= n || i0 >= m) return;
    cplx acc[SMALL_G];
#pragma unroll
    for (int q = 0; q < SMALL_G; q++) acc[q] = mk(0.0, 0.0);
    for (int kk = 0; kk < k; kk++) {
        const cplx b = B[kk + j * ldb];
#pragma unroll
        for (int q = 0; q < SMALL_G; q++)
            if (i0 + q < m) cfma(acc[q], As[kk][i0 + q], b);
    }
    const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
#pragma unroll
    for (int q = 0; q < SMALL_G; q++) {
        if (i0 + q >= m) break;
        const int64_t o = (i0 + q) + j * ldc;
        cplx r = cmul(alpha, acc[q]);
        if (use_beta) r = cadd(r, cmul(beta, C[o]));
        C[o] = r;
    }
}

// Small-dimension dispatch; returns false when the shape is not one of the two forms.
static bool zgemm_small(Context &c, Op opa, Op opb, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda,
                        int64_t sa, const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc,
                        int batch) {
    if (k < 1 || k > SMALL_D) return false;
    if (opa == OP_N && (opb == OP_N || opb == OP_R) && n <= SMALL_D && m >= 64) {
        const int gy = (n + SMALL_G - 1) / SMALL_G;
        const int bx = 256 / gy;   // gy <= 4, bx >= 64
        for (int z0 = 0; z0 < batch; z0 += 65535) {
            const int nz = std::min(65535, batch - z0);
            dim3 grid(grid1d(m, bx), 1, nz), block(bx, gy);
            if (opb == OP_N)
                zgemm_rsmall_kernel<OP_N><<<grid, block, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C,
                                                                        ldc, sc, z0);
            else
                zgemm_rsmall_kernel<OP_R><<<grid, block, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C,
                                                                        ldc, sc, z0);
            DCG_LAUNCHED(c);
        }
        return true;
    }
    if (opa == OP_C && opb == OP_N && m <= SMALL_D && n >= 64) {
        const int gy = (m + SMALL_G - 1) / SMALL_G;
        const int bx = 256 / gy;
        for (int z0 = 0; z0 < batch; z0 += 65535) {
            const int nz = std::min(65535, batch - z0);
            dim3 grid(grid1d(n, bx), 1, nz), block(bx, gy);
            zgemm_lsmall_kernel<<<grid, block, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc,
                                                              z0);
            DCG_LAUNCHED(c);
        }
        return true;
    }
    return false;
}

template <int OPA, int OPB>
static void zgemm_launch(Context &c, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda, int64_t sa,
                         const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc,
                         int batch, int upper, int tile) {
    const int bm = 4 * kZgTyn[tile], bn = 1024 / kZgTyn[tile];
    for (int z0 = 0; z0 < batch; z0 += 65535) {
        int nz = batch - z0 < 65535 ? batch - z0 : 65535;
        dim3 grid(grid1d(m, bm), grid1d(n, bn), nz);
        if (tile == 1)
            zgemm_kernel<OPA, OPB, 8><<<grid, 256, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc,
                                                                  sc, z0, upper);
        else if (tile == 2)
            zgemm_kernel<OPA, OPB, 32><<<grid, 256, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C,
                                                                   ldc, sc, z0, upper);
        else
            zgemm_kernel<OPA, OPB, 16><<<grid, 256, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C,
                                                                   ldc, sc, z0, upper);
        DCG_LAUNCHED(c);
    }
}

// Output tiles of a tile shape (for a Hermitian product's upper half, those touching it).
static int64_t zg_tiles(int m, int n, int tile, int upper) {
    const int bm = 4 * kZgTyn[tile], bn = 1024 / kZgTyn[tile];
    const int64_t tm = (m + bm - 1) / bm, tn = (n + bn - 1) / bn;
    if (!upper) return tm * tn;
    int64_t t = 0;
    for (int64_t j = 0; j < tn; j++) t += std::min<int64_t>(tm, ((j + 1) * bn + bm - 1) / bm);
    return t;
}

// C = alpha * sum_s P_s + beta * C over nsplit partial products (fixed summation order).
__global__ void splitk_reduce_kernel(int m, int n, int nsplit, const cplx *__restrict__ P, cplx alpha, cplx beta,
                                     cplx *C, int64_t ldc, int upper) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t mn = (int64_t)m * n;
    if (idx >= mn) return;
    const int i = (int)(idx % m), j = (int)(idx / m);
    if (upper && i > j) return;
    cplx acc = mk(0.0, 0.0);
    for (int s = 0; s < nsplit; s++) acc = cadd(acc, P[s * mn + idx]);
    const int64_t o = i + (int64_t)j * ldc;
    cplx r = cmul(alpha, acc);
    if (beta.x != 0.0 || beta.y != 0.0) r = cadd(r, cmul(beta, C[o]));
    C[o] = r;
}

template <int OPA, int OPB>
static void zgemm_launch(Context &c, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda, int64_t sa,
                         const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc,
                         int batch, int upper, int tile);
static int64_t zg_tiles(int m, int n, int tile, int upper);

// One split-K product with a given number of K chunks (>= 2): the chunks are computed as one
// batched GEMM into partial products, then reduced in a fixed order.
template <int OPA, int OPB>
static void zgemm_splitk_run(Context &c, int m, int n, int k, int nsplit, cplx alpha, const cplx *A, int64_t lda,
                             const cplx *B, int64_t ldb, cplx beta, cplx *C, int64_t ldc, int upper, int tile) {
    const int kc = (k + nsplit - 1) / nsplit;
    nsplit = (k + kc - 1) / kc;
    const int nfull = k / kc;             // chunks of exactly kc
    const int rem = k - nfull * kc;       // last, shorter chunk
    const int64_t mn = (int64_t)m * n;
    cplx *P = wsget<cplx>(c, "gemm.splitk", (size_t)mn * nsplit);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    // K-chunk strides: A is m x k (OP_N/OP_R, chunk = columns) or k x m (OP_T/OP_C, chunk = rows)
    const int64_t sa = (OPA == OP_N || OPA == OP_R) ? (int64_t)kc * lda : kc;
    const int64_t sb = (OPB == OP_N || OPB == OP_R) ? kc : (int64_t)kc * ldb;
    zgemm_launch<OPA, OPB>(c, m, n, kc, one, A, lda, sa, B, ldb, sb, zero, P, m, mn, nfull, upper, tile);
    if (rem > 0)
        zgemm_launch<OPA, OPB>(c, m, n, rem, one, A + nfull * sa, lda, 0, B + nfull * sb, ldb, 0, zero, P + nfull * mn,
                               m, 0, 1, upper, tile);
    splitk_reduce_kernel<<<grid1d(mn, 256), 256, 0, c.stream>>>(m, n, nsplit, P, alpha, beta, C, ldc, upper);
    DCG_LAUNCHED(c);
}

// The tile shape and K split of one FP64 product.  A GEMM whose output tiles do not fill the
// GPU is split along K into equal chunks of at least 64, computed as one batched GEMM into
// partial products and reduced in a fixed order.  The autotuner times, per shape, every tile
// with no split, with the occupancy heuristic min(2 SMs / tiles, k / 64) and with powers of
// two up to k / 64 (batched products: the tiles alone); candidate 0 (64 x 64 tiles, the
// heuristic split) is used while tuning is off and for calls that accumulate into C (beta
// != 0, which the timed trial runs would disturb).
constexpr double kTuneMinFp64Flops = 1.0e9;

struct ZgPlan {
    int tile, nsplit;
};

static std::vector<ZgPlan> zg_candidates(Context &c, int m, int n, int k, int upper, int batch) {
    const int sms = std::max(1, c.num_sms);
    std::vector<ZgPlan> out;
    for (int t = 0; t < kZgTiles; t++) {
        const int64_t tiles = zg_tiles(m, n, t, upper);
        std::vector<int> ns{1};
        if (batch == 1 && tiles < sms && k >= 128) {
            const int heur = (int)std::min<int64_t>((2 * sms + tiles - 1) / tiles, k / 64);
            if (heur >= 2) ns.insert(ns.begin(), heur);
            for (int p = 2; p <= k / 64 && p <= 64; p *= 2)
                if (std::find(ns.begin(), ns.end(), p) == ns.end()) ns.push_back(p);
        }
        for (int x : ns) out.push_back({t, x});
    }
    return out;
}

template <int OPA, int OPB>
static void zgemm_plan_run(Context &c, const ZgPlan &p, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda,
                           int64_t sa, const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc,
                           int64_t sc, int batch, int upper) {
    if (p.nsplit >= 2) zgemm_splitk_run<OPA, OPB>(c, m, n, k, p.nsplit, alpha, A, lda, B, ldb, beta, C, ldc, upper, p.tile);
    else zgemm_launch<OPA, OPB>(c, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, upper, p.tile);
}

template <int OPA, int OPB>
static void zgemm_tuned(Context &c, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda, int64_t sa,
                        const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc, int batch,
                        int upper) {
    const std::vector<ZgPlan> cand = zg_candidates(c, m, n, k, upper, batch);
    const TuneKey key{TUNE_ZGEMM, OPA * 8 + OPB, m, n, k, upper + 2 * std::min(batch, 1 << 20)};
    // products under ~1 ms of FP64 work keep the heuristic: their trials would cost more than
    // tuning can return (and a served stream meets many shapes once)
    const double work = 8.0 * m * n * (double)k * batch;
    const bool trial_ok = beta.x == 0.0 && beta.y == 0.0 && work >= kTuneMinFp64Flops;
    const int pick = autotune(c, key, (int)cand.size(), trial_ok, [&](int q) {
        zgemm_plan_run<OPA, OPB>(c, cand[q], m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, upper);
    });
    zgemm_plan_run<OPA, OPB>(c, cand[pick], m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, upper);
}

void zgemm(Context &c, Op opa, Op opb, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda, int64_t sa,
           const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc, int batch) {
    if (m <= 0 || n <= 0 || batch <= 0) return;
    GemmTrace trace(c, "fp64", m, n, k, batch);
    if (zgemm_small(c, opa, opb, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch)) return;
#define DCG_ZG(a, b)                                                                                  \
    if (opa == a && opb == b) {                                                                       \
        zgemm_tuned<a, b>(c, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, 0);     \
        return;                                                                                       \
    }
    DCG_ZG(OP_N, OP_N) DCG_ZG(OP_N, OP_T) DCG_ZG(OP_N, OP_C) DCG_ZG(OP_N, OP_R)
    DCG_ZG(OP_T, OP_N) DCG_ZG(OP_T, OP_T) DCG_ZG(OP_T, OP_C) DCG_ZG(OP_T, OP_R)
    DCG_ZG(OP_C, OP_N) DCG_ZG(OP_C, OP_T) DCG_ZG(OP_C, OP_C) DCG_ZG(OP_C, OP_R)
    DCG_ZG(OP_R, OP_N) DCG_ZG(OP_R, OP_T) DCG_ZG(OP_R, OP_C) DCG_ZG(OP_R, OP_R)
#undef DCG_ZG
    throw Error{DCG_E_ARG, "zgemm: bad op"};
}

// Upper triangle of C = A A^H (n x n, A n x k, column-major): only the 64 x 64 tiles on or
// above the diagonal are computed (half the work of the full product), split along k when
// those tiles alone cannot fill the GPU.  The strictly lower part of C is left undefined; a
// Hermitian fill from the upper triangle completes it.
void zherk_upper(Context &c, int n, int k, const cplx *A, int64_t lda, cplx *C, int64_t ldc) {
    if (n <= 0) return;
    GemmTrace trace(c, "herk", n, n, k, 1);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    zgemm_tuned<OP_N, OP_C>(c, n, n, k, one, A, lda, 0, A, lda, 0, zero, C, ldc, 0, 1, 1);
}

// ===================================================================== Hermitian fill
__global__ void herm_from_upper_kernel(int n, cplx *A, int64_t lda) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    int i = (int)(idx % n), j = (int)(idx / n);
    if (i > j) A[i + (int64_t)j * lda] = cconj(A[j + (int64_t)i * lda]);
    else if (i == j) A[i + (int64_t)j * lda].y = 0.0;
}

void herm_from_upper(Context &c, int n, cplx *A, int64_t lda) {
    if (n <= 0) return;
    herm_from_upper_kernel<<<grid1d((int64_t)n * n, 256), 256, 0, c.stream>>>(n, A, lda);
    DCG_LAUNCHED(c);
}

// ===================================================================== deterministic sum
__global__ void dsum_kernel(const double *x, int64_t n, double *out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) *out = s;
}

// Partial sums of contiguous chunks of x (chunk elements each), one block per chunk.
__global__ void dsum_part_kernel(const double *x, int64_t n, int64_t chunk, double *part) {
    __shared__ double sh[32];
    const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(n, lo + chunk);
    double s = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += x[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Sum of x[0..n) into *out.  Long vectors (the per-outer-index E2 terms of F, G and H run to
// millions) are summed in fixed chunks by many blocks, then the chunk sums in order: the order
// depends on n only, so the result is deterministic.
void dsum(Context &c, const double *x, int64_t n, double *out) {
    constexpr int64_t kChunk = 8192;
    if (n <= 4 * kChunk) {
        dsum_kernel<<<1, 1024, 0, c.stream>>>(x, n, out);
        DCG_LAUNCHED(c);
        return;
    }
    const int64_t nb = (n + kChunk - 1) / kChunk;
    double *part = wsget<double>(c, "dsum.part", (size_t)nb);
    dsum_part_kernel<<<(unsigned)nb, 256, 0, c.stream>>>(x, n, kChunk, part);
    DCG_LAUNCHED(c);
    dsum_kernel<<<1, 1024, 0, c.stream>>>(part, nb, out);
    DCG_LAUNCHED(c);
}

void fam_collect(Context &c) {
    for (auto &pr : c.fam_ev) {
        cudaEventSynchronize(pr.second);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pr.first, pr.second);
        c.fam_ms += ms;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    c.fam_ev.clear();
}

// ===================================================================== LU solve
__global__ void lu_pivot_kernel(int n, int k, cplx *A, int64_t lda, int ncols, int *info) {
    __shared__ double best[1024];
    __shared__ int bidx[1024];
    double b = -1.0;
    int bi = k;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
        double a = cabs2(A[i + (int64_t)k * lda]);
        if (a > b) {
            b = a;
            bi = i;
        }
    }
    best[threadIdx.x] = b;
    bidx[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            double o = best[threadIdx.x + s];
            int oi = bidx[threadIdx.x + s];
            if (o > best[threadIdx.x] || (o == best[threadIdx.x] && oi < bidx[threadIdx.x])) {
                best[threadIdx.x] = o;
                bidx[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    const int p = bidx[0];
    if (best[0] == 0.0) {
        if (threadIdx.x == 0 && *info == 0) *info = k + 1;
        return;
    }
    if (p != k)
        for (int j = threadIdx.x; j < ncols; j += blockDim.x) {
            cplx t = A[k + (int64_t)j * lda];
            A[k + (int64_t)j * lda] = A[p + (int64_t)j * lda];
            A[p + (int64_t)j * lda] = t;
        }
    __syncthreads();
    cplx inv = cdiv(mk(1.0, 0.0), A[k + (int64_t)k * lda]);
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (int64_t)k * lda] = cmul(A[i + (int64_t)k * lda], inv);
}

__global__ void lu_update_kernel(int n, int k, cplx *A, int64_t lda, int ncols) {
    const int i = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = k + 1 + blockIdx.y;
    if (i >= n || j >= ncols) return;
    A[i + (int64_t)j * lda] = csub(A[i + (int64_t)j * lda], cmul(A[i + (int64_t)k * lda], A[k + (int64_t)j * lda]));
}

// back substitution U x = y, y in column n of the augmented matrix
__global__ void lu_backsub_kernel(int n, cplx *A, int64_t lda) {
    cplx *b = A + (int64_t)n * lda;
    for (int k = n - 1; k >= 0; k--) {
        __syncthreads();
        cplx xk = cdiv(b[k], A[k + (int64_t)k * lda]);
        __syncthreads();
        if (threadIdx.x == 0) b[k] = xk;
        for (int i = threadIdx.x; i < k; i += blockDim.x) b[i] = csub(b[i], cmul(A[i + (int64_t)k * lda], xk));
    }
}

int zgesv(Context &c, int n, cplx *A, int64_t lda, cplx *b) {
    // augmented copy [A | b]
    cplx *M = wsget<cplx>(c, "gesv.M", (size_t)n * (n + 1));
    int *info = wsget<int>(c, "gesv.info", 1);
    DCG_CUDA(cudaMemcpy2DAsync(M, n * sizeof(cplx), A, lda * sizeof(cplx), n * sizeof(cplx), n,
                               cudaMemcpyDeviceToDevice, c.stream));
    DCG_CUDA(cudaMemcpyAsync(M + (int64_t)n * n, b, n * sizeof(cplx), cudaMemcpyDeviceToDevice, c.stream));
    DCG_CUDA(cudaMemsetAsync(info, 0, sizeof(int), c.stream));
    for (int k = 0; k < n; k++) {
        lu_pivot_kernel<<<1, 1024, 0, c.stream>>>(n, k, M, n, n + 1, info);
        DCG_LAUNCHED(c);
        if (k + 1 < n || true) {
            dim3 g(grid1d(n - k - 1 > 0 ? n - k - 1 : 1, 128), n - k);
            if (n - k - 1 > 0) {
                lu_update_kernel<<<g, 128, 0, c.stream>>>(n, k, M, n, n + 1);
                DCG_LAUNCHED(c);
            }
        }
    }
    lu_backsub_kernel<<<1, 1024, 0, c.stream>>>(n, M, n);
    DCG_LAUNCHED(c);
    DCG_CUDA(cudaMemcpyAsync(b, M + (int64_t)n * n, n * sizeof(cplx), cudaMemcpyDeviceToDevice, c.stream));
    int hinfo = 0;
    DCG_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    return hinfo;
}

}  // namespace dcg
